// sm_103a edge-pull engine: graph build, traversal kernels, drivers, C ABI.
//
// Reference correspondence (stanford-mast/Wedge):
//   build_from_device_edges   graphdata.c:402-585 (vertex index, out-degrees, CSRI)
//   pull_kernel<BFS>          phase_edge_pull_bfs.c:109-332
//   pull_kernel<CC>           phase_edge_pull_cc.c:53-297
//   pull_kernel<SSSP>         phase_edge_pull_sssp.c:57-306
//   pull_kernel<PR>           phase_edge_pull_pr.c:28-116
//   pr_finish_kernel          phases.c:71-114 (ordered merge) + phases.c:37-46 (total rank)
//   pr_vertex_kernel          phase_vertex_pr.c:26-77
//   collect_kernel            wedge.c:63-155 (walk of the active-vertex bitmap)
//   wedge_build_kernel        wedge.c:37-46 (CSRI walk setting frontier bits)
//   decide_kernel             execution_*.c driver loop: mass reduce, dense/Wedge choice, convergence
//   run_traversal / run_pr    execution_{bfs,cc,sssp}.c:122-365 / execution_pr.c:396-486
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <pthread.h>
#include <stdio.h>
#include <time.h>
#include <stdlib.h>
#include <string.h>

#include "engine.cuh"
#include "pull.cuh"
#include "sched.cuh"

namespace wedge {

constexpr int PULL_THREADS = 1024; /* one block per SM: its shared memory holds the hub cache */
constexpr int AUX_THREADS = 256;

int compute_grids(wedge_graph* h);

int cuda_status(cudaError_t e)
{
    if (e == cudaErrorMemoryAllocation)
        return WEDGE_ERR_OOM;
    return WEDGE_ERR_CUDA;
}

int new_handle(wedge_graph** out)
{
    wedge_graph* h = (wedge_graph*)calloc(1, sizeof(wedge_graph));
    if (!h)
        return WEDGE_ERR_OOM;
    h->built_app = -1;
    for (int k = 0; k < WEDGE_KNOBS; ++k)
        h->knob[k] = WEDGE_KNOB_DEFAULT;
    h->last_app = -1;
    h->graph_app = -1;
    h->pend_app = -1;
    WEDGE_CHECK(cudaGetDevice(&h->device));
    WEDGE_CHECK(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device));
    WEDGE_CHECK(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking));
    h->stream = h->own_stream;
    for (int i = 0; i < 8; ++i)
        WEDGE_CHECK(cudaEventCreate(&h->ev[i]));
    WEDGE_CHECK(cudaEventCreateWithFlags(&h->ev_run, cudaEventDisableTiming));
    WEDGE_CHECK(cudaEventCreateWithFlags(&h->ev_x, cudaEventDisableTiming));
    WEDGE_CHECK(cudaMallocHost((void**)&h->h_ctrl, sizeof(Ctrl)));
    h->iter_pull_ms = (double*)calloc(LOG_CAP, sizeof(double));
    h->iter_wedge_ms = (double*)calloc(LOG_CAP, sizeof(double));
    if (!h->iter_pull_ms || !h->iter_wedge_ms)
        return WEDGE_ERR_OOM;
    *out = h;
    return WEDGE_OK;
}

int track(wedge_graph* h, void* p)
{
    if (h->nallocs >= (int)(sizeof(h->allocs) / sizeof(h->allocs[0])))
        return WEDGE_ERR_OOM;
    h->allocs[h->nallocs++] = p;
    return WEDGE_OK;
}

static int track_state(wedge_graph* h, void* p)
{
    if (h->nstate >= (int)(sizeof(h->state_allocs) / sizeof(h->state_allocs[0])))
        return WEDGE_ERR_OOM;
    h->state_allocs[h->nstate++] = p;
    return WEDGE_OK;
}

static void free_state(wedge_graph* h)
{
    for (int i = 0; i < h->nstate; ++i)
        cudaFree(h->state_allocs[i]);
    h->nstate = 0;
    memset(&h->s, 0, sizeof(h->s));
    h->s.net = h->net; /* the scheduler network outlives the state arrays */
    h->built_app = -1;
    h->cc_pending = 0;
    if (h->graph_exec) {
        cudaGraphExecDestroy(h->graph_exec);
        h->graph_exec = nullptr;
        h->graph_app = -1;
    }
    if (h->pr_exec) {
        cudaGraphExecDestroy(h->pr_exec);
        h->pr_exec = nullptr;
    }
}

void free_handle(wedge_graph* h)
{
    if (!h)
        return;
    if (h->stream)
        cudaStreamSynchronize(h->stream);
    if (h->xstream)
        cudaStreamSynchronize(h->xstream);
    free_state(h);
    for (int i = 0; i < h->nallocs; ++i)
        cudaFree(h->allocs[i]);
    for (int i = 0; i < 8; ++i)
        if (h->ev[i])
            cudaEventDestroy(h->ev[i]);
    if (h->h_ctrl)
        cudaFreeHost(h->h_ctrl);
    if (h->net)
        cudaFree(h->net);
    free(h->iter_pull_ms);
    free(h->iter_wedge_ms);
    if (h->ev_run)
        cudaEventDestroy(h->ev_run);
    if (h->ev_x)
        cudaEventDestroy(h->ev_x);
    if (h->xstream)
        cudaStreamDestroy(h->xstream);
    if (h->xbuf)
        cudaFree(h->xbuf);
    if (h->own_stream)
        cudaStreamDestroy(h->own_stream); /* a caller's stream stays the caller's */
    free(h);
}

template <class T>
static int dalloc(wedge_graph* h, T** p, uint64_t count, bool state = false)
{
    *p = nullptr;
    const size_t bytes = (size_t)(count ? count : 1) * sizeof(T);
    cudaError_t e = cudaMalloc((void**)p, bytes);
    if (e != cudaSuccess)
        return cuda_status(e);
    return state ? track_state(h, *p) : track(h, *p);
}

static uint32_t grid_for(uint64_t work, uint32_t threads, uint32_t cap)
{
    uint64_t b = (work + threads - 1) / threads;
    if (b < 1)
        b = 1;
    return (uint32_t)(b < cap ? b : cap);
}

/* ================================================================= build */

__global__ void validate_kernel(const uint32_t* src, const uint32_t* dst, uint64_t E, uint64_t V, int* err)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t d = dst[e];
        if (src[e] >= V || d >= V)
            atomicOr(err, 1);
        if (e > 0 && dst[e - 1] > d)
            atomicOr(err, 2);
    }
}

// head flag of edge e: first in-edge of its destination (graphdata.c:402-427)
__global__ void head_flag_kernel(const uint32_t* dst, uint64_t E, uint32_t* flag)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x)
        flag[e] = (e == 0 || dst[e] != dst[e - 1]) ? 1u : 0u;
}

// kidx = inclusive scan of head flags: compressed destination = kidx - 1
__global__ void compress_kernel(const uint32_t* dst, const uint32_t* kidx, uint64_t E, uint32_t* dst_id,
                                unsigned long long* dst_off)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        if (e == 0 || dst[e] != dst[e - 1]) {
            const uint32_t k = kidx[e] - 1u;
            dst_id[k] = dst[e];
            dst_off[k] = e;
        }
    }
}

__global__ void tile_index_kernel(const uint32_t* kidx, uint64_t E, uint32_t T, uint32_t Vne, uint32_t* tile_dst0,
                                  unsigned long long* dst_off)
{
    for (uint64_t t = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; t <= T; t += (uint64_t)gridDim.x * blockDim.x) {
        tile_dst0[t] = (t * TILE < E) ? kidx[t * TILE] - 1u : Vne; /* padding edges: no owner */
        if (t == 0)
            dst_off[Vne] = E;
    }
}

__global__ void outdeg_kernel(const uint32_t* src, uint64_t E, uint32_t* outdeg)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x)
        atomicAdd(&outdeg[src[e]], 1u);
}

__global__ void widen_kernel(const uint32_t* in, unsigned long long* out, uint64_t n)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = in[i];
}

// CSRI fill (graphdata.c:535-569), grouped by source: the in-edge position of
// every out-edge (its chunk is position / 32), or, on graphs whose padded
// in-edges do not fit 32 bits, its chunk id
__global__ void csri_fill_kernel(const uint32_t* src, uint64_t E, unsigned long long* cursor, uint32_t* csri,
                                 uint32_t positions)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long pos = atomicAdd(&cursor[src[e]], 1ull);
        csri[pos] = (uint32_t)(positions ? e : e / CHUNK);
    }
}

// bit dst_off[k] of the destination-start bitmap, for every compressed destination
__global__ void dst_start_kernel(const unsigned long long* dst_off, uint32_t num_dsts, uint32_t* start)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < num_dsts; k += gridDim.x * blockDim.x) {
        const unsigned long long p = dst_off[k];
        atomicOr(&start[p >> 5], 1u << (uint32_t)(p & 31u));
    }
}

// Destinations whose in-edges span tiles, for the PageRank merge: those spanning
// at most SPLIT_SERIAL tile boundaries from the front of the lists (count[0]),
// the longer ones from the back (count[1]; entry cap-1-j).  Every split holds a
// distinct tile boundary, so the two ends never meet in lists of T entries.
constexpr uint32_t SPLIT_SERIAL = 8;
__global__ void split_kernel(const unsigned long long* dst_off, uint32_t Vne, uint32_t cap, uint32_t tile, uint32_t* split_k,
                             uint32_t* split_t0, uint32_t* split_t1, unsigned int* count)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < Vne; k += gridDim.x * blockDim.x) {
        const uint32_t t0 = (uint32_t)(dst_off[k] / tile);
        const uint32_t t1 = (uint32_t)((dst_off[k + 1] - 1) / tile);
        if (t0 != t1) {
            const unsigned int i = t1 - t0 <= SPLIT_SERIAL ? atomicAdd(&count[0], 1u) : cap - 1u - atomicAdd(&count[1], 1u);
            split_k[i] = k;
            split_t0[i] = t0;
            split_t1[i] = t1;
        }
    }
}

// vertex -> compressed destination index (preset to NONE32: no in-edges)
__global__ void dst_index_kernel(const uint32_t* dst_id, uint32_t Vne, uint32_t* inv)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < Vne; k += gridDim.x * blockDim.x)
        inv[dst_id[k]] = k;
}

// Symmetry: the reverse of every edge s -> d is an edge, i.e. d is among the
// in-neighbours of s (ascending within a destination: a binary search).  Sets
// *asym at the first edge without its reverse; the others then stop early.
__global__ void sym_check_kernel(const uint32_t* src, const uint32_t* dst, uint64_t E, const uint32_t* inv,
                                 const unsigned long long* dst_off, unsigned int* asym)
{
    uint32_t n = 0;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        if ((++n & 63u) == 0u && *(volatile unsigned int*)asym)
            return;
        const uint32_t sv = src[e], d = dst[e];
        const uint32_t k = inv[sv];
        bool found = false;
        if (k != NONE32) {
            unsigned long long lo = dst_off[k], hi = dst_off[k + 1]; /* first source >= d in [lo, hi) */
            while (lo < hi) {
                const unsigned long long mid = lo + (hi - lo) / 2u;
                if (src[mid] < d)
                    lo = mid + 1u;
                else
                    hi = mid;
            }
            found = lo < dst_off[k + 1] && src[lo] == d;
        }
        if (!found) {
            atomicOr(asym, 1u);
            return;
        }
    }
}

// largest weight word (uint64 weights; the byte-wide copy applies below 256)
__global__ void max_weight_kernel(const unsigned long long* w, uint64_t E, unsigned long long* out)
{
    unsigned long long m = 0;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x)
        m = w[e] > m ? w[e] : m;
    for (int d = 16; d > 0; d >>= 1) {
        const unsigned long long y = __shfl_xor_sync(FULL, m, d);
        m = y > m ? y : m;
    }
    if ((threadIdx.x & 31) == 0 && m)
        atomicMax(out, m);
}

__global__ void narrow_weights_kernel(const unsigned long long* w, uint64_t Epad, uint8_t* w8)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < Epad; e += (uint64_t)gridDim.x * blockDim.x)
        w8[e] = (uint8_t)w[e];
}

__global__ void pad_kernel(uint32_t* src, unsigned long long* w, uint64_t E, uint64_t Epad)
{
    for (uint64_t e = E + blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < Epad; e += (uint64_t)gridDim.x * blockDim.x) {
        src[e] = NONE32;
        if (w)
            w[e] = 0ull;
    }
}

template <class InT, class OutT>
static int device_scan(wedge_graph* h, const InT* in, OutT* out, uint64_t n, bool inclusive)
{
    size_t bytes = 0;
    if (inclusive)
        WEDGE_CHECK(cub::DeviceScan::InclusiveSum(nullptr, bytes, in, out, (long long)n, h->stream));
    else
        WEDGE_CHECK(cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, (long long)n, h->stream));
    void* tmp = nullptr;
    WEDGE_CHECK(cudaMallocAsync(&tmp, bytes, h->stream));
    cudaError_t e = inclusive ? cub::DeviceScan::InclusiveSum(tmp, bytes, in, out, (long long)n, h->stream)
                              : cub::DeviceScan::ExclusiveSum(tmp, bytes, in, out, (long long)n, h->stream);
    cudaFreeAsync(tmp, h->stream);
    WEDGE_CHECK(e);
    return WEDGE_OK;
}

// key of vertex v for the degree order: descending out-degree, then ascending id
__global__ void degree_key_kernel(const uint32_t* outdeg, uint64_t V, unsigned long long* key)
{
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x)
        key[v] = ((unsigned long long)(~outdeg[v]) << 32) | (unsigned long long)v;
}

__global__ void permutation_kernel(const unsigned long long* sorted_key, uint64_t V, uint32_t* new2old, uint32_t* old2new)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < V; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t old = (uint32_t)(sorted_key[i] & 0xffffffffull);
        new2old[i] = old;
        old2new[old] = (uint32_t)i;
    }
}

__global__ void relabel_edges_kernel(const uint32_t* src, const uint32_t* dst, uint64_t E, const uint32_t* old2new,
                                     unsigned long long* key)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x)
        key[e] = ((unsigned long long)old2new[dst[e]] << 32) | old2new[src[e]];
}

__global__ void unpack_edges_kernel(const unsigned long long* key, uint64_t E, uint32_t* src, uint32_t* dst)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        src[e] = (uint32_t)(key[e] & 0xffffffffull);
        dst[e] = (uint32_t)(key[e] >> 32);
    }
}

// Degree relabelling: vertices are renumbered by descending out-degree (ties
// by id), so the sources gathered most often are the lowest ids and share cache
// lines; edges are renumbered and re-sorted by (destination, source).  The
// permutations stay on the device: roots are mapped in, results mapped back.
static int relabel_by_degree(wedge_graph* h, uint64_t V, uint64_t E, uint32_t* d_src, uint32_t* d_dst,
                             unsigned long long* d_w, uint32_t** new2old, uint32_t** old2new,
                             const uint32_t* global_outdeg)
{
    cudaStream_t st = h->stream;
    const uint32_t cap = (uint32_t)h->num_sms * 16u;
    int rc;
    if ((rc = dalloc(h, new2old, V)) || (rc = dalloc(h, old2new, V)))
        return rc;
    uint32_t* deg = nullptr;
    unsigned long long *vk = nullptr, *vk2 = nullptr;
    WEDGE_CHECK(cudaMallocAsync((void**)&deg, V * sizeof(uint32_t), st));
    WEDGE_CHECK(cudaMallocAsync((void**)&vk, V * sizeof(unsigned long long), st));
    WEDGE_CHECK(cudaMallocAsync((void**)&vk2, V * sizeof(unsigned long long), st));
    if (global_outdeg) { /* a shard: the whole graph's degrees, so every shard numbers vertices alike */
        WEDGE_CHECK(cudaMemcpyAsync(deg, global_outdeg, V * sizeof(uint32_t), cudaMemcpyDeviceToDevice, st));
    } else {
        WEDGE_CHECK(cudaMemsetAsync(deg, 0, V * sizeof(uint32_t), st));
        if (E)
            outdeg_kernel<<<grid_for(E, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(d_src, E, deg);
    }
    degree_key_kernel<<<grid_for(V, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(deg, V, vk);
    {
        cub::DoubleBuffer<unsigned long long> db(vk, vk2);
        size_t tb = 0;
        WEDGE_CHECK(cub::DeviceRadixSort::SortKeys(nullptr, tb, db, (long long)V, 0, 64, st));
        void* tmp = nullptr;
        WEDGE_CHECK(cudaMallocAsync(&tmp, tb ? tb : 1, st));
        WEDGE_CHECK(cub::DeviceRadixSort::SortKeys(tmp, tb, db, (long long)V, 0, 64, st));
        cudaFreeAsync(tmp, st);
        permutation_kernel<<<grid_for(V, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(db.Current(), V, *new2old, *old2new);
    }
    cudaFreeAsync(deg, st);
    cudaFreeAsync(vk, st);
    cudaFreeAsync(vk2, st);
    if (E == 0)
        return WEDGE_OK;
    int vbits = 1;
    while (vbits < 32 && (1ull << vbits) < V)
        ++vbits;
    unsigned long long *ek = nullptr, *ek2 = nullptr, *w2 = nullptr;
    WEDGE_CHECK(cudaMallocAsync((void**)&ek, E * sizeof(unsigned long long), st));
    WEDGE_CHECK(cudaMallocAsync((void**)&ek2, E * sizeof(unsigned long long), st));
    relabel_edges_kernel<<<grid_for(E, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(d_src, d_dst, E, *old2new, ek);
    cub::DoubleBuffer<unsigned long long> kb(ek, ek2);
    size_t tb = 0;
    void* tmp = nullptr;
    if (d_w) {
        WEDGE_CHECK(cudaMallocAsync((void**)&w2, E * sizeof(unsigned long long), st));
        cub::DoubleBuffer<unsigned long long> vb(d_w, w2);
        WEDGE_CHECK(cub::DeviceRadixSort::SortPairs(nullptr, tb, kb, vb, (long long)E, 0, 32 + vbits, st));
        WEDGE_CHECK(cudaMallocAsync(&tmp, tb ? tb : 1, st));
        WEDGE_CHECK(cub::DeviceRadixSort::SortPairs(tmp, tb, kb, vb, (long long)E, 0, 32 + vbits, st));
        if (vb.Current() != d_w)
            WEDGE_CHECK(cudaMemcpyAsync(d_w, vb.Current(), E * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st));
    } else {
        WEDGE_CHECK(cub::DeviceRadixSort::SortKeys(nullptr, tb, kb, (long long)E, 0, 32 + vbits, st));
        WEDGE_CHECK(cudaMallocAsync(&tmp, tb ? tb : 1, st));
        WEDGE_CHECK(cub::DeviceRadixSort::SortKeys(tmp, tb, kb, (long long)E, 0, 32 + vbits, st));
    }
    unpack_edges_kernel<<<grid_for(E, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(kb.Current(), E, d_src, d_dst);
    cudaFreeAsync(tmp, st);
    cudaFreeAsync(ek, st);
    cudaFreeAsync(ek2, st);
    if (w2)
        cudaFreeAsync(w2, st);
    WEDGE_CHECK(cudaGetLastError());
    return WEDGE_OK;
}

// Builds the device CSC from destination-sorted device edge arrays.  d_src and
// d_w (if any) must hold roundup(E, TILE) entries and become owned by the
// handle; d_dst is consumed and freed.
__global__ void permute_degrees_kernel(const uint32_t* global_outdeg, const uint32_t* new2old, uint64_t V, uint32_t* outdeg)
{
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < V; v += (uint64_t)gridDim.x * blockDim.x)
        outdeg[v] = global_outdeg[new2old[v]];
}

// Builds the device CSC.  A shard (d_global_outdeg given: the whole graph's
// out-degrees, caller numbering) numbers vertices by those degrees, so all
// shards share one numbering, and keeps them as its out-degrees (the changed
// mass and PageRank's divisor), while its CSRI indexes its own in-edges.
int build_from_device_edges(wedge_graph* h, uint64_t V, uint64_t E, uint32_t* d_src, uint32_t* d_dst,
                            unsigned long long* d_w, int weight_kind, const uint32_t* d_global_outdeg)
{
    cudaStream_t st = h->stream;
    DevGraph& g = h->g;
    g.V = V;
    g.E = E;
    g.E_thr = E;
    g.Epad = (E + MAX_TILE_E - 1) / MAX_TILE_E * MAX_TILE_E;
    g.T = (uint32_t)(g.Epad / TILE);
    g.weight_kind = (uint32_t)weight_kind;
    h->weight_kind = weight_kind;
    g.src = d_src;
    g.w = d_w;
    const uint32_t cap = (uint32_t)h->num_sms * 16u;

    int* d_err = nullptr;
    WEDGE_CHECK(cudaMallocAsync((void**)&d_err, sizeof(int), st));
    WEDGE_CHECK(cudaMemsetAsync(d_err, 0, sizeof(int), st));
    if (E)
        validate_kernel<<<grid_for(E, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(d_src, d_dst, E, V, d_err);
    int herr = 0;
    WEDGE_CHECK(cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, st));
    WEDGE_CHECK(cudaStreamSynchronize(st));
    cudaFreeAsync(d_err, st);
    if (herr) {
        cudaFreeAsync(d_dst, st);
        return WEDGE_ERR_FORMAT;
    }
    {
        uint32_t *n2o = nullptr, *o2n = nullptr;
        int rc = relabel_by_degree(h, V, E, d_src, d_dst, d_w, &n2o, &o2n, d_global_outdeg);
        if (rc)
            return rc;
        g.new2old = n2o;
        g.old2new = o2n;
    }

    // compressed destinations
    uint32_t* kidx = nullptr;
    WEDGE_CHECK(cudaMallocAsync((void**)&kidx, (E ? E : 1) * sizeof(uint32_t), st));
    uint32_t Vne = 0;
    if (E) {
        head_flag_kernel<<<grid_for(E, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(d_dst, E, kidx);
        int rc = device_scan(h, kidx, kidx, E, true);
        if (rc)
            return rc;
        WEDGE_CHECK(cudaMemcpyAsync(&Vne, kidx + (E - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
        WEDGE_CHECK(cudaStreamSynchronize(st));
    }
    g.Vne = Vne;
    uint32_t *dst_id, *tile_dst0, *outdeg, *csri;
    unsigned long long *dst_off, *csri_off;
    int rc;
    if ((rc = dalloc(h, &dst_id, Vne)) || (rc = dalloc(h, &dst_off, (uint64_t)Vne + 1)) ||
        (rc = dalloc(h, &tile_dst0, (uint64_t)g.T + 1)) || (rc = dalloc(h, &outdeg, V)) ||
        (rc = dalloc(h, &csri_off, V + 1)) || (rc = dalloc(h, &csri, E)))
        return rc;
    if (E) {
        compress_kernel<<<grid_for(E, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(d_dst, kidx, E, dst_id, dst_off);
    }
    tile_index_kernel<<<grid_for((uint64_t)g.T + 1, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(kidx, E, g.T, Vne,
                                                                                               tile_dst0, dst_off);
    // symmetry (CC's label space)
    unsigned int h_asym = 1u;
    if (E) {
        uint32_t* inv = nullptr;
        unsigned int* d_asym = nullptr;
        WEDGE_CHECK(cudaMallocAsync((void**)&inv, V * sizeof(uint32_t), st));
        WEDGE_CHECK(cudaMallocAsync((void**)&d_asym, sizeof(unsigned int), st));
        WEDGE_CHECK(cudaMemsetAsync(d_asym, 0, sizeof(unsigned int), st));
        WEDGE_CHECK(cudaMemsetAsync(inv, 0xFF, V * sizeof(uint32_t), st));
        dst_index_kernel<<<grid_for(Vne, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(dst_id, Vne, inv);
        sym_check_kernel<<<grid_for(E, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(d_src, d_dst, E, inv, dst_off, d_asym);
        WEDGE_CHECK(cudaMemcpyAsync(&h_asym, d_asym, sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
        cudaFreeAsync(d_asym, st);
        cudaFreeAsync(inv, st);
    }
    cudaFreeAsync(kidx, st);
    cudaFreeAsync(d_dst, st);

    // out-degrees and CSRI: in-edge positions where they fit 32 bits
    // (WEDGE_CSRI_CHUNKS=1 selects chunk ids on any graph: the encoding, and
    // the chunk Wedge pulls, of graphs beyond 2^32 padded in-edges)
    const char* force_chunks = getenv("WEDGE_CSRI_CHUNKS");
    const uint32_t csri_pos = (g.Epad < (1ull << 32) && !(force_chunks && force_chunks[0] == '1')) ? 1u : 0u;
    WEDGE_CHECK(cudaMemsetAsync(outdeg, 0, V * sizeof(uint32_t), st));
    if (E)
        outdeg_kernel<<<grid_for(E, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(d_src, E, outdeg);
    unsigned long long* wide = nullptr;
    WEDGE_CHECK(cudaMallocAsync((void**)&wide, (V + 1) * sizeof(unsigned long long), st));
    widen_kernel<<<grid_for(V, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(outdeg, wide, V);
    WEDGE_CHECK(cudaMemsetAsync(wide + V, 0, sizeof(unsigned long long), st));
    if ((rc = device_scan(h, wide, csri_off, V + 1, false)))
        return rc;
    WEDGE_CHECK(cudaMemcpyAsync(wide, csri_off, (V + 1) * sizeof(unsigned long long), cudaMemcpyDeviceToDevice, st));
    if (E)
        csri_fill_kernel<<<grid_for(E, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(d_src, E, wide, csri, csri_pos);
    cudaFreeAsync(wide, st);
    if (d_global_outdeg) /* the shard's own counts built the CSRI; the graph's degrees from here on */
        permute_degrees_kernel<<<grid_for(V, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(d_global_outdeg, g.new2old, V, outdeg);

    // destination starts, one bit per in-edge (the pulls' tile geometry)
    uint32_t* dst_start = nullptr;
    const uint64_t start_words = g.Epad / 32 + 1;
    if ((rc = dalloc(h, &dst_start, start_words)))
        return rc;
    WEDGE_CHECK(cudaMemsetAsync(dst_start, 0, start_words * sizeof(uint32_t), st));
    if (Vne)
        dst_start_kernel<<<grid_for(Vne, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(dst_off, Vne, dst_start);

    // destinations whose in-edges span tiles (PageRank fixup list)
    uint32_t *split_k, *split_t0, *split_t1;
    if ((rc = dalloc(h, &split_k, g.T)) || (rc = dalloc(h, &split_t0, g.T)) || (rc = dalloc(h, &split_t1, g.T)))
        return rc;
    unsigned int* d_cnt = nullptr;
    WEDGE_CHECK(cudaMallocAsync((void**)&d_cnt, 2 * sizeof(unsigned int), st));
    WEDGE_CHECK(cudaMemsetAsync(d_cnt, 0, 2 * sizeof(unsigned int), st));
    if (Vne)
        split_kernel<<<grid_for(Vne, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(dst_off, Vne, g.T, TILE, split_k, split_t0,
                                                                             split_t1, d_cnt);
    unsigned int nsplit[2] = {0, 0};
    WEDGE_CHECK(cudaMemcpyAsync(nsplit, d_cnt, 2 * sizeof(unsigned int), cudaMemcpyDeviceToHost, st));
    // dst_id ascends, so it is the identity when its last entry is Vne-1 (symmetric
    // graphs after the degree relabelling: in-degree > 0 exactly for ids < Vne)
    uint32_t last_dst = 0;
    if (Vne)
        WEDGE_CHECK(cudaMemcpyAsync(&last_dst, dst_id + (Vne - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    if (g.Epad > E)
        pad_kernel<<<1, 128, 0, st>>>(d_src, d_w, E, g.Epad);
    WEDGE_CHECK(cudaStreamSynchronize(st));
    cudaFreeAsync(d_cnt, st);
    WEDGE_CHECK(cudaGetLastError());
    g.nsplit = nsplit[0];
    g.nwide = nsplit[1];
    // SSSP weights in one byte each where every uint64 weight is below 256: the
    // pulls stream 1 byte per in-edge instead of 8 (same arithmetic, 64-bit sums)
    g.w8 = nullptr;
    if (d_w && weight_kind == WEDGE_WEIGHTS_U64 && E) {
        unsigned long long* d_max = nullptr;
        unsigned long long wmax = 0;
        WEDGE_CHECK(cudaMallocAsync((void**)&d_max, sizeof(unsigned long long), st));
        WEDGE_CHECK(cudaMemsetAsync(d_max, 0, sizeof(unsigned long long), st));
        max_weight_kernel<<<grid_for(E, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(d_w, E, d_max);
        WEDGE_CHECK(cudaMemcpyAsync(&wmax, d_max, sizeof(wmax), cudaMemcpyDeviceToHost, st));
        WEDGE_CHECK(cudaStreamSynchronize(st));
        cudaFreeAsync(d_max, st);
        if (wmax < 256ull) {
            uint8_t* w8 = nullptr;
            if ((rc = dalloc(h, &w8, g.Epad)))
                return rc;
            narrow_weights_kernel<<<grid_for(g.Epad, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(d_w, g.Epad, w8);
            WEDGE_CHECK(cudaGetLastError());
            g.w8 = w8;
        }
    }
    g.dst_ident = (Vne && last_dst == Vne - 1) ? 1u : 0u;
    g.sym = h_asym ? 0u : 1u;
    g.dst_id = dst_id;
    g.dst_off = dst_off;
    g.tile_dst0 = tile_dst0;
    g.dst_start = dst_start;
    g.outdeg = outdeg;
    g.csri_off = csri_off;
    g.csri = csri;
    g.csri_pos = csri_pos;
    g.split_k = split_k;
    g.split_t0 = split_t0;
    g.split_t1 = split_t1;

    return compute_grids(h);
}

/* ============================================================ traversal */

__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long x)
{
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
        x += __shfl_xor_sync(FULL, x, d);
    return x;
}

__device__ __forceinline__ double warp_sum_f64(double x)
{
#pragma unroll
    for (int d = 16; d > 0; d >>= 1)
        x = __dadd_rn(x, __shfl_xor_sync(FULL, x, d));
    return x;
}

__device__ __forceinline__ const uint32_t* cur_front(const DevState& s, uint32_t parity)
{
    return parity ? s.front1 : s.front0;
}

// pull output bitmap: the other half of the double buffer.  The pull reads the
// vertices the previous pull activated (BFS frontier; CC/SSSP changed
// vertices, read by the source-filtered pull) and writes the ones it activates.
__device__ __forceinline__ uint32_t* next_front(const DevState& s, uint32_t parity)
{
    return parity ? s.front0 : s.front1;
}

// in-edges per lane of each application's pull (tile = 32 * EPL in-edges)
template <int APP>
struct PullEpl {
    static constexpr int value = 8;
};
#ifndef WEDGE_EPL_CC
#define WEDGE_EPL_CC 16
#endif
template <>
struct PullEpl<WEDGE_APP_CC> {
    static constexpr int value = WEDGE_EPL_CC;
};
template <>
struct PullEpl<WEDGE_APP_PR> {
    static constexpr int value = 4; /* the PageRank split lists are built for 128-edge tiles */
};

// One tile's bounds, loaded one tile ahead of its processing so their latency
// overlaps the previous tile's work.
struct TileIn {
    uint32_t t, cmask, k0, kend, visw;
    bool open;     // some destination of the tile is not finished
    bool anydone;  // some destination of the tile is finished (its in-edges need no gathers)
};

template <int APP, int EPL>
__device__ __forceinline__ void tile_prefetch(const DevGraph& g, const DevState& s, uint32_t t, uint32_t cmask, int lane,
                                              TileIn& in)
{
    constexpr uint32_t Q = EPL / 4; /* 128-edge index entries per tile */
    in.t = t;
    in.cmask = cmask;
    in.k0 = g.tile_dst0[(uint64_t)t * Q];
    in.kend = g.tile_dst0[((uint64_t)t + 1) * Q];
    in.open = true;
    in.anydone = false;
    in.visw = 0u;
    if (APP == WEDGE_APP_BFS || APP == WEDGE_APP_CC) {
        // skip a tile whose destinations are all finished: visited (BFS; the
        // reference's jump over converged vertices, phase_edge_pull_bfs.c:189-204)
        // or holding label 0, the smallest label there is (CC)
        const uint32_t klim = min(in.kend, g.Vne - 1u);
        const uint32_t w0 = in.k0 >> 5, w1 = klim >> 5;
        bool open = false, done = false;
        uint32_t visw = 0u;
        if ((uint32_t)lane <= w1 - w0) {
            const uint32_t wi = w0 + lane;
            const uint32_t lo = (wi == w0) ? (in.k0 & 31u) : 0u;
            const uint32_t hi = (wi == w1) ? (klim & 31u) : 31u;
            const uint32_t range = (hi == 31u ? FULL : ((2u << hi) - 1u)) & ~((1u << lo) - 1u);
            visw = s.vis_c[wi];
            open = (~visw & range) != 0u;
            done = (visw & range) != 0u;
        }
        in.visw = visw;
        in.open = __any_sync(FULL, open);
        in.anydone = __any_sync(FULL, done);
        if (s.tile_open && !in.open && lane == 0)
            atomicAnd(&s.tile_open[t >> 5], ~(1u << (t & 31u))); /* closed for good */
    }
}

// EPL consecutive sources of this lane (positions EPL*lane ..), NONE32 where the
// lane's chunk is not in the mask.  Whole 32-byte sectors per lane (256-bit
// loads) for EPL >= 8, one 128-bit load for EPL = 4: each sector of the tile
// is requested once, with no reliance on L1 reuse.
template <int EPL>
__device__ __forceinline__ void load_sources(const DevGraph& g, uint64_t base, uint32_t cmask, int lane,
                                             uint32_t (&sa)[EPL], unsigned long long pol)
{
    const bool on = (cmask >> (((uint32_t)lane * EPL) >> 5)) & 1u;
    const uint32_t* p = g.src + base + (uint64_t)lane * EPL;
    if constexpr (EPL % 8 == 0) {
#pragma unroll
        for (int q = 0; q < EPL / 8; ++q) {
            uint32_t x[8];
            if (on) {
                ld_stream_v8_ef(p + 8 * q, x, pol);
            } else {
#pragma unroll
                for (int j = 0; j < 8; ++j)
                    x[j] = NONE32;
            }
#pragma unroll
            for (int j = 0; j < 8; ++j)
                sa[8 * q + j] = x[j];
        }
    } else {
#pragma unroll
        for (int q = 0; q < EPL / 4; ++q) {
            uint4 x = make_uint4(NONE32, NONE32, NONE32, NONE32);
            if (on)
                x = __ldg(reinterpret_cast<const uint4*>(p) + q);
            sa[4 * q + 0] = x.x;
            sa[4 * q + 1] = x.y;
            sa[4 * q + 2] = x.z;
            sa[4 * q + 3] = x.w;
        }
    }
}

// The tiles a warp pulls: every tile (dense: static stride, or for BFS the open
// tiles, 32 per dynamically grabbed word of the open-tile bitmap), or the tiles
// of the Wedge frontier from the list compact_kernel built.  Warp-uniform.
struct TileIter {
    uint32_t i, step;      // dense (static stride), the probe's tile list, or the Wedge list
    uint32_t tbeg, tend;   // the tiles [tbeg, tend) of this launch (CC's hub / other split)
    bool need;             // walk the tiles the probe listed (dense BFS/CC pulls, candidate pulls)
};

template <int APP, int EPL>
__device__ __forceinline__ bool next_tile(const DevGraph& g, const DevState& s, uint32_t mode, uint32_t t_end,
                                          TileIter& it, int lane, uint32_t& t, uint32_t& cmask)
{
    constexpr uint32_t MASK = (EPL >= 32) ? FULL : ((1u << EPL) - 1u);
    // dense BFS/CC pulls (and candidate Wedge pulls) walk the list of tiles their
    // probe left work in (tile_list, each tile once); a CC launch takes the
    // ones of its range
    if (it.need) {
        const uint32_t n = s.ctrl->need_n;
        for (;;) {
            if (it.i >= n)
                return false;
            t = (uint32_t)(s.tile_list[it.i] >> 32);
            it.i += it.step;
            if (t >= it.tbeg && t < it.tend)
                break;
        }
        cmask = MASK;
        return true;
    }
    if (mode != MODE_WEDGE) {
        if (it.i >= t_end)
            return false;
        t = it.i;
        cmask = MASK;
        it.i += it.step;
        return true;
    }
    // Wedge: the (tile, chunk mask) list compact_kernel built from the frontier
    const uint32_t n = s.ctrl->tiles;
    if (it.i >= n)
        return false;
    const unsigned long long e = s.tile_list[it.i];
    it.i += it.step;
    t = (uint32_t)(e >> 32);
    cmask = (uint32_t)e & MASK;
    return true;
}

template <int APP>
struct CurT {
    using type = uint32_t;
};
template <>
struct CurT<WEDGE_APP_SSSP> {
    using type = unsigned long long;
};

// bounded mbarrier probes before a pull gives up on its hub-cache copy
constexpr uint32_t HUB_WAIT_TRIES = 1u << 20;
enum : uint32_t { ERR_HUB_TIMEOUT = 2u };

// pull phases: 0 = all tiles; CC/SSSP dense pulls run as two launches,
// 1 = tiles [0, hub_tile) (the hub destinations), 2 = tiles [hub_tile, T),
// so the second launch caches hub values that no tile of it can change.
// dst_kernel phases before a dense pull: A = the BFS or CC probe, or the hub
// destinations of CC's first pull over engine ids; B = the other destinations
// of that first pull (CC)
enum : uint32_t { PHASE_ALL = 0, PHASE_HUBS = 1, PHASE_REST = 2, PHASE_DST_A = 3, PHASE_DST_B = 4 };

__host__ __device__ constexpr bool two_phase_app(int app)
{
    return app == WEDGE_APP_CC || app == WEDGE_APP_SSSP;
}

// launches of one pull (each fills its own NCNT block counters per block):
// PageRank: tiles; BFS: dst_kernel A + tiles; CC: dst_kernel A and B + hub
// tiles + other tiles; SSSP: hub tiles + other tiles
__host__ __device__ constexpr uint32_t pull_launches_of(int app)
{
    return app == WEDGE_APP_PR ? 1u : app == WEDGE_APP_CC ? 4u : 2u;
}
// dst_kernel launches of one pull
__host__ __device__ constexpr uint32_t dst_launches_of(int app)
{
    return app == WEDGE_APP_BFS ? 1u : app == WEDGE_APP_CC ? 2u : 0u;
}

// SSSP narrow distances: a distance write, recorded in the 32-bit copy the
// pulls gather (4 bytes per gather instead of 8).  The copy holds distances
// below narrow_lim (2^32-1, or a smaller limit that tests set), NONE32 for the
// others; distances only decrease, so the copy is never below the distance.
// A finite distance at or above the limit sets Ctrl::narrow_ovf, after which
// the pulls gather the 64-bit distances from their next launch on (a source a
// pull skipped as unreached meanwhile changed in this iteration: the next pull
// relaxes it).
__device__ __forceinline__ void dist32_put(const DevState& s, uint32_t v, unsigned long long d, bool sole)
{
    if (!s.dist32)
        return;
    if (d >= (unsigned long long)s.narrow_lim) {
        atomicOr(&s.ctrl->narrow_ovf, 1u);
        return;
    }
    if (sole)
        s.dist32[v] = (uint32_t)d;
    else
        atomicMin(&s.dist32[v], (uint32_t)d);
}

// The Wedge pull of SSSP over in-edge positions: every vertex the last pull
// activated relaxes exactly the in-edges its out-edges are (the CSRI holds
// their positions), where the chunk form pulls the whole 32-edge chunks
// holding them (phase_edge_pull_sssp.c:171-306 over the chunks
// wedge_generate_frontier marks).  Both reach the same fixed point, the least
// dist[d] = min over in-edges of dist[s] + w, by monotone relaxations; only
// the iteration counts may differ.  Vertices with at most BIG_LIST out-edges
// take a thread each; expand_kernel split the longer lists into PIECE-entry
// items, which take a warp each.  block_cnt as pull_kernel's.
__device__ __forceinline__ void sssp_push_pull(const DevGraph& g, const DevState& s, const Ctrl* c,
                                               unsigned long long* block_cnt)
{
    constexpr int WARPS = PULL_THREADS / 32;
    __shared__ unsigned long long sh_pc[WARPS][4];
    __shared__ unsigned int sh_pdeg[3];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    uint32_t* nxt = next_front(s, c->parity);
    const bool f64 = g.weight_kind == WEDGE_WEIGHTS_F64;
    unsigned long long mass = 0, edges = 0, act = 0, occ = 0;
    if (threadIdx.x < 3)
        sh_pdeg[threadIdx.x] = 0u;
    __syncthreads();
    auto relax = [&](unsigned long long du, uint32_t pos) {
        const unsigned long long wv = g.w8 ? (unsigned long long)g.w8[pos] : g.w[pos];
        const unsigned long long nd =
            f64 ? (unsigned long long)__double_as_longlong(__dadd_rn(__longlong_as_double((long long)du),
                                                                     __longlong_as_double((long long)wv)))
                : du + wv; /* phase_edge_pull_sssp.c:136-137; an activated source is reached */
        const uint32_t k = dst_of_pos(g, pos);
        const uint32_t vtx = g.dst_ident ? k : g.dst_id[k];
        if (nd < s.prop64[vtx] && nd < atomicMin(&s.prop64[vtx], nd)) {
            dist32_put(s, vtx, nd, false);
            const uint32_t b = 1u << (vtx & 31u);
            const uint32_t o = atomicOr(&nxt[vtx >> 5], b);
            occ += o == 0u ? 1u : 0u;
            if (!(o & b)) {
                const uint32_t od = g.outdeg[vtx];
                mass += od;
                ++act;
                const uint32_t bk = degree_bucket(od);
                if (bk < 3u)
                    atomicAdd(&sh_pdeg[bk], 1u);
            }
        }
    };
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthr = gridDim.x * blockDim.x;
    const uint32_t n = c->alist_n;
    for (uint32_t i = tid; i < n; i += nthr) {
        const uint32_t u = s.alist[i];
        const unsigned long long lo = g.csri_off[u], len = g.csri_off[u + 1u] - lo;
        if (len > BIG_LIST)
            continue; /* an item of expand_kernel's */
        const unsigned long long du = s.prop64[u];
        uint32_t pos[BIG_LIST];
#pragma unroll
        for (uint32_t j = 0; j < BIG_LIST; ++j)
            pos[j] = (j < len) ? g.csri[lo + j] : 0u;
#pragma unroll
        for (uint32_t j = 0; j < BIG_LIST; ++j)
            if (j < len)
                relax(du, pos[j]);
        edges += len;
    }
    const uint32_t ni = c->items;
    for (uint32_t i = tid >> 5; i < ni; i += nthr >> 5) {
        const uint2 it = s.items[i];
        const unsigned long long lo = g.csri_off[it.x] + (unsigned long long)it.y * PIECE;
        const unsigned long long end = g.csri_off[it.x + 1u];
        const unsigned long long hi = (lo + PIECE < end) ? lo + PIECE : end;
        const unsigned long long du = s.prop64[it.x];
        for (unsigned long long j = lo + (unsigned long long)lane; j < hi; j += 32u) {
            relax(du, g.csri[j]);
            ++edges;
        }
    }
    mass = warp_sum_u64(mass);
    edges = warp_sum_u64(edges);
    act = warp_sum_u64(act);
    occ = warp_sum_u64(occ);
    if (lane == 0) {
        sh_pc[wib][0] = mass;
        sh_pc[wib][1] = edges;
        sh_pc[wib][2] = act;
        sh_pc[wib][3] = occ;
    }
    __syncthreads();
    if (threadIdx.x < NCNT) {
        unsigned long long a = 0;
        const int col = threadIdx.x == CNT_MASS ? 0 : threadIdx.x == CNT_EDGES ? 1 : threadIdx.x == CNT_ACT ? 2
                      : threadIdx.x == CNT_OCC ? 3 : -1;
        if (col >= 0)
            for (int w = 0; w < WARPS; ++w)
                a += sh_pc[w][col];
        if (threadIdx.x >= CNT_DEG0 && threadIdx.x <= CNT_DEG2)
            a = sh_pdeg[threadIdx.x - CNT_DEG0];
        block_cnt[NCNT * blockIdx.x + threadIdx.x] = a;
    }
}

// BFS/CC probe: in-edges of an unfinished destination read before the tile pull
// (the default of Ctrl::probe_edges; the probe-window knob overrides it)
constexpr uint32_t PROBE_EDGES = 16;

// Edge pull over all tiles (dense) or over the tiles of the Wedge frontier.
// block_cnt[NCNT*b + CNT_*] = changed mass, in-edges read, tiles visited,
// destinations in visited tiles, vertices activated.
// One 1024-thread block per SM; dynamic shared memory holds the hub cache:
// elements [0, s.hub_n) of the gathered array (BFS frontier words, CC labels,
// SSSP distances, PageRank ranks), bulk-copied at the start of the launch.
// Warps start on global memory and switch to the cache once its copy landed.
template <int APP, int EPL>
__global__ void __launch_bounds__(PULL_THREADS, 1)
    pull_kernel(DevGraph g, DevState s, unsigned long long* block_cnt, uint32_t phase)
{
    constexpr int WARPS = PULL_THREADS / 32;
    constexpr uint32_t TILE_E = 32u * EPL;
    constexpr uint32_t TAB = 129; /* staged destinations per tile; more are read from global memory */
    using cur_t = typename CurT<APP>::type;
    __shared__ unsigned long long sh_cnt[WARPS][NCNT];
    __shared__ uint32_t tab_id[WARPS][TAB];  // vertex id of each destination of the warp's tile
    __shared__ cur_t tab_cur[WARPS][TAB];    // its property before the tile (min apps)
    __shared__ unsigned long long hub_bar;
    __shared__ unsigned int sh_deg[3];
    extern __shared__ __align__(16) unsigned char hub_smem[];
    Ctrl* c = s.ctrl;
    if (c->done)
        return;
    const uint32_t mode = c->mode;
    if (phase == PHASE_REST && mode == MODE_WEDGE) {
        // a Wedge pull runs whole in the first launch: this one only reports zeros
        if (threadIdx.x < NCNT)
            block_cnt[NCNT * blockIdx.x + threadIdx.x] = 0ull;
        return;
    }
    if (APP == WEDGE_APP_SSSP && mode == MODE_WEDGE && s.push) {
        sssp_push_pull(g, s, c, block_cnt);
        return;
    }
    /* the in-edge stream is read once per pull: it should not push the gathered array out of L2 */
    const unsigned long long pol = l2_evict_first_policy();
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t T = (uint32_t)((g.E + TILE_E - 1) / TILE_E); /* tiles holding real in-edges */
    uint32_t t_begin = 0, t_end = T;
    if (two_phase_app(APP) && mode != MODE_WEDGE) {
        const uint32_t split = min(s.hub_tile, T);
        if (phase == PHASE_HUBS)
            t_end = split;
        else
            t_begin = split;
    }
    const uint32_t parity = c->parity;
    const uint32_t* cur = cur_front(s, parity);
    const bool filtered = (APP == WEDGE_APP_CC || APP == WEDGE_APP_SSSP) && mode == MODE_FILTERED;
    uint32_t* nxt = next_front(s, parity);
    uint32_t* my_id = tab_id[wib];
    cur_t* my_cur = tab_cur[wib];
    unsigned long long mass = 0, edges = 0, tiles = 0, dsts = 0, act = 0, occ = 0;
    auto count_act = [&](uint32_t d) {
        mass += d;
        ++act;
        const uint32_t b = degree_bucket(d);
        if (b < 3u)
            atomicAdd(&sh_deg[b], 1u); /* activated vertices per out-degree bucket 0..2 */
    };
    auto vid = [&](uint32_t k, uint32_t slot) -> uint32_t { return slot < TAB ? my_id[slot] : g.dst_id[k]; };

    // ---- hub cache
    // SSSP gathers the 32-bit copy of the distances while every distance fits
    const bool narrow = APP == WEDGE_APP_SSSP && s.dist32 && !c->narrow_ovf;
    const bool wide = (APP == WEDGE_APP_SSSP && !narrow) || (APP == WEDGE_APP_PR); /* FP32C PageRank: pr32_pull_kernel */
    const void* hub_src = (APP == WEDGE_APP_BFS)    ? (const void*)cur
                          : (APP == WEDGE_APP_CC)   ? (const void*)s.prop32
                          : (APP == WEDGE_APP_SSSP) ? (narrow ? (const void*)s.dist32 : (const void*)s.prop64)
                                                    : (const void*)s.rank;
    const uint64_t hub_have = ((APP == WEDGE_APP_BFS) ? (g.V + 31) / 32 : g.V) * (wide ? 8u : 4u);
    const uint64_t hub_fit = hub_have & ~15ull;
    const uint32_t hub_bytes = (uint64_t)s.hub_bytes < hub_fit ? s.hub_bytes : (uint32_t)hub_fit; /* within smem and the array */
    bool use_hub = hub_bytes != 0u && ((uintptr_t)hub_src & 15u) == 0u && (smem_u32(hub_smem) & 15u) == 0u;
    if (APP == WEDGE_APP_BFS)
        use_hub = use_hub && (mode != MODE_WEDGE || c->tiles >= T / 16u);
    else if (two_phase_app(APP))
        use_hub = use_hub && mode != MODE_WEDGE;
    if (APP == WEDGE_APP_SSSP && s.dist32 && !narrow)
        use_hub = false; /* the cache is sized and split for the 32-bit copy */
    uint32_t* hub32 = reinterpret_cast<uint32_t*>(hub_smem);
    unsigned long long* hub64 = reinterpret_cast<unsigned long long*>(hub_smem);
    if (threadIdx.x < 3)
        sh_deg[threadIdx.x] = 0u;
    __syncthreads();
    if (use_hub) {
        if (threadIdx.x == 0) {
            mbar_init(&hub_bar, 1u);
            mbar_arrive_expect_tx(&hub_bar, hub_bytes);
            for (uint32_t off = 0; off < hub_bytes; off += 32768u)
                bulk_g2s(hub_smem + off, static_cast<const unsigned char*>(hub_src) + off, min(32768u, hub_bytes - off),
                         &hub_bar);
        }
        __syncthreads();
    }
    uint32_t hub_lim = 0; /* elements of the cache this warp reads: 0 until the copy completed */

    TileIter it;
    it.need = s.tile_need && (mode == MODE_DENSE || (mode == MODE_WEDGE && s.cand));
    it.i = it.need ? gw : t_begin + gw; /* the probe's list starts at 0 */
    it.step = nw;
    it.tbeg = t_begin;
    it.tend = t_end;
    TileIn nextin;
    uint32_t tn, cn;
    bool more = next_tile<APP, EPL>(g, s, mode, t_end, it, lane, tn, cn);
    if (more)
        tile_prefetch<APP, EPL>(g, s, tn, cn, lane, nextin);
    while (more) {
        const TileIn in = nextin;
        more = next_tile<APP, EPL>(g, s, mode, t_end, it, lane, tn, cn);
        if (more)
            tile_prefetch<APP, EPL>(g, s, tn, cn, lane, nextin);
        ++tiles;
        if (!in.open)
            continue;
        if (use_hub && hub_lim == 0u) {
            uint32_t ready = 0u;
            if (lane == 0)
                ready = mbar_test_wait(&hub_bar, 0u) ? 1u : 0u;
            if (__shfl_sync(FULL, ready, 0))
                hub_lim = hub_bytes / (wide ? 8u : 4u);
        }
        const uint32_t t = in.t;
        const uint64_t base = (uint64_t)t * TILE_E;
        const bool last_tile = (t + 1u >= T);
        uint32_t sa[EPL];
        load_sources<EPL>(g, base, in.cmask, lane, sa, pol);
#pragma unroll
        for (int q = 0; q < EPL; ++q)
            edges += (sa[q] != NONE32) ? 1u : 0u;

        if (APP == WEDGE_APP_BFS) {
            // Frontier-bit gathers.  A tile with no visited destination gathers at
            // once (the latency overlaps the geometry's); otherwise the geometry
            // comes first and only the in-edges of unvisited destinations gather.
            // ids of the tile's first 32 destinations: loaded now, staged after the gathers
            const uint32_t nst = min(min(in.kend, g.Vne - 1u) - in.k0 + 1u, TAB);
            uint32_t st_id = 0u;
            if ((uint32_t)lane < nst)
                st_id = g.dst_ident ? in.k0 + (uint32_t)lane : g.dst_id[in.k0 + (uint32_t)lane];
            uint32_t v[EPL];
            auto gather = [&](uint32_t x) -> uint32_t {
                const uint32_t wi = x >> 5; /* NONE32 >> 5 lies beyond any cache */
                const uint32_t fb = (wi < hub_lim) ? hub32[wi] : ((x != NONE32) ? ld_ro_u32(cur + wi) : 0u);
                return ((fb >> (x & 31u)) & 1u) ? x : NONE32;
            };
            if (!in.anydone) {
#pragma unroll
                for (int q = 0; q < EPL; ++q)
                    v[q] = gather(sa[q]);
            }
            TileGeo<EPL> tg;
            tile_geometry_bits<EPL>(g, base, last_tile, in.k0, in.kend, lane, tg);
            dsts += tg.ndst;
            if (in.anydone) {
                const uint32_t w0 = in.k0 >> 5;
#pragma unroll
                for (int q = 0; q < EPL; ++q) {
                    const uint32_t k = pos_dst(tg, q);
                    const uint32_t vw = __shfl_sync(FULL, in.visw, (int)((k >> 5) - w0));
                    v[q] = gather(((vw >> (k & 31u)) & 1u) ? NONE32 : sa[q]);
                }
            }
            if ((uint32_t)lane < nst)
                my_id[lane] = st_id;
            for (uint32_t slot = (uint32_t)lane + 32u; slot < min(tg.ndst, TAB); slot += 32u)
                my_id[slot] = g.dst_id[tg.k0 + slot];
            __syncwarp();
            seg_reduce<EPL>(v, tg, lane, MinU32(), [&](uint32_t k, uint32_t val, int kind) {
                if (val == NONE32)
                    return;
                const uint32_t vtx = vid(k, k - tg.k0);
                // a destination whose in-edges all lie in this tile has no other
                // writer in this pull, and it was unvisited when the tile began
                const uint32_t old = (kind == EMIT_COMPLETE) ? (s.prop32[vtx] = val, NONE32) : atomicMin(&s.prop32[vtx], val);
                if (old == NONE32) {
                    atomicOr(&s.vis_c[k >> 5], 1u << (k & 31u));
                    occ += atomicOr(&nxt[vtx >> 5], 1u << (vtx & 31u)) == 0u ? 1u : 0u;
                    count_act(g.outdeg[vtx]);
                }
            });
        } else if (APP == WEDGE_APP_CC) {
            // Label gathers.  A tile whose destinations all may still drop gathers at
            // once (the latency overlaps the geometry's); otherwise the geometry
            // comes first and destinations holding label 0 gather nothing.
            // the tile's first 32 destinations: ids and labels loaded now, staged after the gathers
            const uint32_t nst = min(min(in.kend, g.Vne - 1u) - in.k0 + 1u, TAB);
            uint32_t st_id = 0u;
            if ((uint32_t)lane < nst)
                st_id = g.dst_ident ? in.k0 + (uint32_t)lane : g.dst_id[in.k0 + (uint32_t)lane];
            uint32_t v[EPL];
            auto gather = [&](uint32_t x) -> uint32_t {
                if (filtered && x != NONE32 && !((ld_ro_u32(cur + (x >> 5)) >> (x & 31u)) & 1u))
                    return NONE32; /* source unchanged by the previous pull */
                return (x < hub_lim) ? hub32[x] : ((x != NONE32) ? s.prop32[x] : NONE32);
            };
            if (!in.anydone) {
#pragma unroll
                for (int q = 0; q < EPL; ++q)
                    v[q] = gather(sa[q]);
            }
            TileGeo<EPL> tg;
            tile_geometry_bits<EPL>(g, base, last_tile, in.k0, in.kend, lane, tg);
            dsts += tg.ndst;
            if (in.anydone) {
                const uint32_t w0 = in.k0 >> 5;
#pragma unroll
                for (int q = 0; q < EPL; ++q) {
                    const uint32_t k = pos_dst(tg, q);
                    const uint32_t vw = __shfl_sync(FULL, in.visw, (int)((k >> 5) - w0));
                    v[q] = gather(((vw >> (k & 31u)) & 1u) ? NONE32 : sa[q]);
                }
            }
            if ((uint32_t)lane < nst) {
                my_id[lane] = st_id;
                my_cur[lane] = s.prop32[st_id];
            }
            for (uint32_t slot = (uint32_t)lane + 32u; slot < min(tg.ndst, TAB); slot += 32u) {
                const uint32_t vtx = g.dst_id[tg.k0 + slot];
                my_id[slot] = vtx;
                my_cur[slot] = s.prop32[vtx];
            }
            __syncwarp();
            seg_reduce<EPL>(v, tg, lane, MinU32(), [&](uint32_t k, uint32_t val, int kind) {
                const uint32_t slot = k - tg.k0;
                const uint32_t vtx = vid(k, slot);
                const uint32_t cv = slot < TAB ? (uint32_t)my_cur[slot] : s.prop32[vtx];
                if (val < cv) {
                    if (vtx < hub_lim)
                        atomicMin(&hub32[vtx], val); /* keeps this block's cache current (hub phase) */
                    if (val == 0u)
                        atomicOr(&s.vis_c[k >> 5], 1u << (k & 31u)); /* label 0 is final */
                    const uint32_t b = 1u << (vtx & 31u);
                    if (kind == EMIT_COMPLETE) {
                        // sole writer of vtx in this launch: cv is current; the
                        // probe may have set its changed bit already
                        s.prop32[vtx] = val;
                        const uint32_t o = atomicOr(&nxt[vtx >> 5], b);
                        occ += o == 0u ? 1u : 0u;
                        if (!(o & b))
                            count_act(g.outdeg[vtx]);
                    } else if (val < atomicMin(&s.prop32[vtx], val)) {
                        const uint32_t o = atomicOr(&nxt[vtx >> 5], b);
                        occ += o == 0u ? 1u : 0u;
                        if (!(o & b))
                            count_act(g.outdeg[vtx]);
                    }
                }
            });
        } else if (APP == WEDGE_APP_SSSP) {
            unsigned long long wv[EPL];
            const bool on = (in.cmask >> (((uint32_t)lane * EPL) >> 5)) & 1u;
            if (g.w8) { /* byte-wide weights: EPL bytes per lane (SSSP's EPL is a multiple of 8) */
#pragma unroll
                for (int q = 0; q < EPL / 8; ++q) {
                    const unsigned long long x =
                        on ? ld_stream_u64_ef(g.w8 + base + (uint64_t)lane * EPL + 8 * q, pol) : 0ull;
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        wv[8 * q + j] = (x >> (8 * j)) & 0xFFull;
                }
            } else {
                const unsigned long long* wp = g.w + base + (uint64_t)lane * EPL;
#pragma unroll
                for (int q = 0; q < EPL / 4; ++q) {
                    unsigned long long x[4] = {0ull, 0ull, 0ull, 0ull};
                    if (on)
                        ld_stream_v4u64_ef(wp + 4 * q, x, pol);
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        wv[4 * q + j] = x[j];
                }
            }
            unsigned long long v[EPL];
#pragma unroll
            for (int q = 0; q < EPL; ++q) {
                v[q] = NONE64;
                if (sa[q] != NONE32 && (!filtered || ((ld_ro_u32(cur + (sa[q] >> 5)) >> (sa[q] & 31u)) & 1u))) {
                    unsigned long long d;
                    if (narrow) {
                        const uint32_t x = (sa[q] < hub_lim) ? hub32[sa[q]] : ld_gather_u32(s.dist32 + sa[q]);
                        d = (x == NONE32) ? NONE64 : (unsigned long long)x;
                    } else {
                        d = (sa[q] < hub_lim) ? hub64[sa[q]] : s.prop64[sa[q]];
                    }
                    if (g.weight_kind == WEDGE_WEIGHTS_F64)
                        v[q] = (unsigned long long)__double_as_longlong(
                            __dadd_rn(__longlong_as_double((long long)d), __longlong_as_double((long long)wv[q])));
                    else
                        v[q] = (d == NONE64) ? NONE64 : d + wv[q]; /* phase_edge_pull_sssp.c:136-137 */
                }
            }
            TileGeo<EPL> tg;
            tile_geometry_bits<EPL>(g, base, last_tile, in.k0, in.kend, lane, tg);
            dsts += tg.ndst;
            for (uint32_t slot = (uint32_t)lane; slot < min(tg.ndst, TAB); slot += 32u) {
                const uint32_t vtx = g.dst_ident ? tg.k0 + slot : g.dst_id[tg.k0 + slot];
                my_id[slot] = vtx;
                if (narrow) { /* exact while no distance reached 2^32-1 (dist32_put) */
                    const uint32_t x = s.dist32[vtx];
                    my_cur[slot] = (x == NONE32) ? NONE64 : (unsigned long long)x;
                } else {
                    my_cur[slot] = s.prop64[vtx];
                }
            }
            __syncwarp();
            seg_reduce<EPL>(v, tg, lane, MinU64(), [&](uint32_t k, unsigned long long val, int kind) {
                const uint32_t slot = k - tg.k0;
                const uint32_t vtx = vid(k, slot);
                const unsigned long long cv = slot < TAB ? (unsigned long long)my_cur[slot] : s.prop64[vtx];
                if (val < cv) {
                    if (vtx < hub_lim) {
                        if (narrow)
                            atomicMin(&hub32[vtx], val < (unsigned long long)s.narrow_lim ? (uint32_t)val : NONE32);
                        else
                            atomicMin(&hub64[vtx], val);
                    }
                    const uint32_t b = 1u << (vtx & 31u);
                    if (kind == EMIT_COMPLETE) {
                        s.prop64[vtx] = val; /* sole writer, as for CC: the bit is new */
                        dist32_put(s, vtx, val, true);
                        atomicOr(&nxt[vtx >> 5], b);
                        ++occ;
                        count_act(g.outdeg[vtx]);
                    } else if (val < atomicMin(&s.prop64[vtx], val)) {
                        dist32_put(s, vtx, val, false);
                        const uint32_t o = atomicOr(&nxt[vtx >> 5], b);
                        occ += o == 0u ? 1u : 0u;
                        if (!(o & b))
                            count_act(g.outdeg[vtx]);
                    }
                }
            });
        } else if (APP == WEDGE_APP_PR) {
            double v[EPL];
#pragma unroll
            for (int q = 0; q < EPL; ++q)
                v[q] = (sa[q] < hub_lim)    ? reinterpret_cast<const double*>(hub_smem)[sa[q]]
                       : (sa[q] != NONE32) ? ld_ro_f64(s.rank + sa[q])
                                           : 0.0;
            TileGeo<EPL> tg;
            tile_geometry_bits<EPL>(g, base, last_tile, in.k0, in.kend, lane, tg);
            dsts += tg.ndst;
            for (uint32_t slot = (uint32_t)lane; slot < min(tg.ndst, TAB); slot += 32u)
                my_id[slot] = g.dst_ident ? tg.k0 + slot : g.dst_id[tg.k0 + slot];
            __syncwarp();
            seg_reduce<EPL>(v, tg, lane, AddF64(), [&](uint32_t k, double val, int kind) {
                if (kind == EMIT_COMPLETE)
                    s.acc[vid(k, k - tg.k0)] = val;
                else if (kind == EMIT_HEAD)
                    s.head_part[t] = val;
                else
                    s.tail_part[t] = val;
            });
        }
        __syncwarp(); /* the table is rewritten by the next tile */
    }
    // the block may not retire with its bulk copy in flight
    if (use_hub && threadIdx.x == 0 && !mbar_wait_bounded(&hub_bar, 0u, HUB_WAIT_TRIES)) {
        atomicOr(&c->error, ERR_HUB_TIMEOUT);
        mbar_wait_bounded(&hub_bar, 0u, HUB_WAIT_TRIES);
    }
    // per-block counters (no same-address atomics): reduced by decide_kernel
    mass = warp_sum_u64(mass);
    edges = warp_sum_u64(edges);
    act = warp_sum_u64(act);
    occ = warp_sum_u64(occ);
    if (lane == 0) {
        sh_cnt[wib][CNT_MASS] = mass;
        sh_cnt[wib][CNT_EDGES] = edges;
        sh_cnt[wib][CNT_TILES] = tiles;  // warp-uniform
        sh_cnt[wib][CNT_DSTS] = dsts;    // warp-uniform
        sh_cnt[wib][CNT_ACT] = act;
        sh_cnt[wib][CNT_DEG0] = 0ull;
        sh_cnt[wib][CNT_DEG1] = 0ull;
        sh_cnt[wib][CNT_DEG2] = 0ull;
        sh_cnt[wib][CNT_OCC] = occ;
    }
    __syncthreads();
    if (threadIdx.x < NCNT) {
        unsigned long long a = 0;
        for (int w = 0; w < WARPS; ++w)
            a += sh_cnt[w][threadIdx.x];
        if (threadIdx.x >= CNT_DEG0 && threadIdx.x <= CNT_DEG2)
            a = sh_deg[threadIdx.x - CNT_DEG0];
        block_cnt[NCNT * blockIdx.x + threadIdx.x] = a;
    }
}

// SSSP dense and source-filtered pulls over 512-edge tiles, for graphs with
// byte-wide weights and in-edge positions in the CSRI (Wedge pulls relax the
// activated sources' in-edges, sssp_push_pull).  Lane l loads its 16 sources
// (two 256-bit loads) and 16 weight bytes (one 128-bit load), gathers the
// sources' distances (hub cache or global memory) and adds the weights; the
// warp takes the per-destination minimum with the segmented reduction.  The
// minima of the tile's first complete destinations (256 with 32-bit sums, 128
// with 64-bit ones) are staged
// in the warp's slice of shared memory and compared, written and activated by
// the warp's lanes together over consecutive destinations; spanning
// destinations take atomicMin.  While the distances fit the 32-bit copy the
// candidates are 32-bit sums (a sum at or above the copy's limit is dropped,
// Ctrl::narrow_ovf and Ctrl::ovf_redo are set, and the next pull is a dense
// 64-bit one, which relaxes every in-edge again).  Two instantiations run
// each launch, the 64-bit one first: SUMS32 for dense and filtered pulls while
// the distances fit the copy, the other for the rest (and the Wedge pulls);
// each returns at once where the other runs (the 32-bit one may set
// Ctrl::narrow_ovf, so it runs second).  Two launches as pull_kernel's (hub
// destinations' tiles first).  Dynamic shared memory: hub cache | staged minima.
constexpr int SSSP_EPL = 16;
constexpr uint32_t SSSP_TILE = 32u * SSSP_EPL;
constexpr uint32_t SSSP_SLOTS = 128;   /* staged 64-bit minima per warp (64-bit instantiation) */
constexpr uint32_t SSSP_SLOTS32 = 256; /* staged 32-bit minima per warp: the tiles with more destinations
                                          (R-MAT scale 22: 7% of the complete ones, 25% past 128 slots) */
constexpr uint32_t SSSP_WARP_STAGE = SSSP_SLOTS * 8u > SSSP_SLOTS32 * 4u ? SSSP_SLOTS * 8u : SSSP_SLOTS32 * 4u;
constexpr uint32_t SSSP_STAGE_BYTES = (PULL_THREADS / 32) * SSSP_WARP_STAGE;

template <bool SUMS32>
__global__ void __launch_bounds__(PULL_THREADS, 1)
    sssp_pull_kernel(DevGraph g, DevState s, unsigned long long* block_cnt, uint32_t phase)
{
    constexpr int EPL = SSSP_EPL;
    constexpr int WARPS = PULL_THREADS / 32;
    constexpr uint32_t Q = SSSP_TILE / TILE;
    __shared__ unsigned long long sh_cnt[WARPS][NCNT];
    __shared__ unsigned long long hub_bar;
    __shared__ unsigned int sh_deg[3];
    extern __shared__ __align__(16) unsigned char sssp_smem[];
    Ctrl* c = s.ctrl;
    if (c->done)
        return;
    const uint32_t mode = c->mode;
    if ((mode != MODE_WEDGE && s.dist32 && !c->narrow_ovf && s.narrow_sums) != SUMS32)
        return; /* the other instantiation's launch */
    if (mode == MODE_WEDGE) {
        if (phase == PHASE_HUBS)
            sssp_push_pull(g, s, c, block_cnt);
        else if (threadIdx.x < NCNT)
            block_cnt[NCNT * blockIdx.x + threadIdx.x] = 0ull; /* a Wedge pull runs whole in the first launch */
        return;
    }
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t T = (uint32_t)((g.E + SSSP_TILE - 1) / SSSP_TILE);
    const uint32_t split = min(s.hub_tile, T);
    const uint32_t t_begin = phase == PHASE_HUBS ? 0u : split, t_end = phase == PHASE_HUBS ? split : T;
    const uint32_t* cur = cur_front(s, c->parity);
    uint32_t* nxt = next_front(s, c->parity);
    const bool filtered = mode == MODE_FILTERED;
    const uint32_t hub_bytes = s.hub_bytes;
    const bool narrow = s.dist32 && !c->narrow_ovf; /* gathers from the 32-bit copy (and, SUMS32, sums) */
    const uint32_t lim = s.narrow_lim;
    bool dropped = false;                           /* a 32-bit sum reached the limit */
    const unsigned long long pol = l2_evict_first_policy(); /* for the in-edge and weight streams */
    const unsigned char* hub_src = narrow ? reinterpret_cast<const unsigned char*>(s.dist32)
                                          : reinterpret_cast<const unsigned char*>(s.prop64);
    uint32_t* hub32 = reinterpret_cast<uint32_t*>(sssp_smem);
    unsigned long long* hub64 = reinterpret_cast<unsigned long long*>(sssp_smem);
    constexpr uint32_t SLOTS = SUMS32 ? SSSP_SLOTS32 : SSSP_SLOTS;
    unsigned char* stage = sssp_smem + hub_bytes + (uint32_t)wib * SSSP_WARP_STAGE;
    uint32_t* my_min32 = reinterpret_cast<uint32_t*>(stage);
    unsigned long long* my_min64 = reinterpret_cast<unsigned long long*>(stage);
    unsigned long long mass = 0, edges = 0, tiles = 0, dsts = 0, act = 0, occ = 0;
    if (threadIdx.x < 3)
        sh_deg[threadIdx.x] = 0u;
    /* the cache is sized and split for the 32-bit copy where there is one */
    const bool use_hub = hub_bytes != 0u && ((uintptr_t)hub_src & 15u) == 0u && (narrow || !s.dist32);
    __syncthreads();
    if (use_hub) {
        if (threadIdx.x == 0) {
            mbar_init(&hub_bar, 1u);
            mbar_arrive_expect_tx(&hub_bar, hub_bytes);
            for (uint32_t off = 0; off < hub_bytes; off += 32768u)
                bulk_g2s(sssp_smem + off, hub_src + off, min(32768u, hub_bytes - off), &hub_bar);
        }
        __syncthreads();
    }
    uint32_t hub_lim = 0;
    // a destination's distance before this launch (the 32-bit copy is exact
    // while no distance reached 2^32-1)
    auto cur_dist = [&](uint32_t vtx) -> unsigned long long {
        if (narrow) {
            const uint32_t x = s.dist32[vtx];
            return x == NONE32 ? NONE64 : (unsigned long long)x;
        }
        return s.prop64[vtx];
    };
    auto hub_min = [&](uint32_t vtx, unsigned long long val) {
        if (vtx >= hub_lim)
            return;
        if (narrow)
            atomicMin(&hub32[vtx], val < (unsigned long long)lim ? (uint32_t)val : NONE32);
        else
            atomicMin(&hub64[vtx], val);
    };
    // activated vertices per out-degree bucket 0..2, packed 21 bits each per lane
    unsigned long long degs = 0;
    auto count_deg = [&](uint32_t od) {
        const uint32_t bk = degree_bucket(od);
        if (bk < 3u)
            degs += 1ull << (21u * bk);
    };
    // a changed destination: its bit in the next frontier and, the first time, its out-edge mass
    auto activate = [&](uint32_t vtx) {
        const uint32_t b = 1u << (vtx & 31u);
        const uint32_t o = atomicOr(&nxt[vtx >> 5], b);
        occ += o == 0u ? 1u : 0u;
        if (!(o & b)) {
            const uint32_t od = g.outdeg[vtx];
            mass += od;
            ++act;
            count_deg(od);
        }
    };
    // the same for a destination this launch writes once (its bit is new)
    auto activate_new = [&](uint32_t vtx) {
        atomicOr(&nxt[vtx >> 5], 1u << (vtx & 31u));
        ++occ;
        const uint32_t od = g.outdeg[vtx];
        mass += od;
        ++act;
        count_deg(od);
    };
    uint32_t t = t_begin + gw;
    uint32_t k0n = 0, kendn = 0;
    if (t < t_end) {
        k0n = g.tile_dst0[(uint64_t)t * Q];
        kendn = g.tile_dst0[((uint64_t)t + 1u) * Q];
    }
    for (; t < t_end; t += nw) {
        const uint32_t k0 = k0n, kend = kendn;
        if (t + nw < t_end) {
            k0n = g.tile_dst0[(uint64_t)(t + nw) * Q];
            kendn = g.tile_dst0[((uint64_t)(t + nw) + 1u) * Q];
        }
        if (use_hub && hub_lim == 0u) {
            uint32_t ready = 0u;
            if (lane == 0)
                ready = mbar_test_wait(&hub_bar, 0u) ? 1u : 0u;
            if (__shfl_sync(FULL, ready, 0))
                hub_lim = hub_bytes / (narrow ? 4u : 8u);
        }
        ++tiles;
        const uint64_t base = (uint64_t)t * SSSP_TILE;
        uint32_t sa[EPL];
        {
            const uint32_t* p = g.src + base + (uint64_t)lane * EPL;
            uint32_t x[8];
            ld_stream_v8_ef(p, x, pol);
#pragma unroll
            for (int j = 0; j < 8; ++j)
                sa[j] = x[j];
            ld_stream_v8_ef(p + 8, x, pol);
#pragma unroll
            for (int j = 0; j < 8; ++j)
                sa[8 + j] = x[j];
        }
        const uint4 wq = ld_stream_v4u32_ef(g.w8 + base + (uint64_t)lane * EPL, pol);
        const uint32_t wword[4] = {wq.x, wq.y, wq.z, wq.w};
        if (lane == 0) /* in-edges of the tile: all but the padding after the last one */
            edges += (g.E - base < SSSP_TILE) ? g.E - base : SSSP_TILE;
        // a tile minimum the reduction ends: staged (the tile's first SLOTS
        // complete destinations, which the lanes then compare and write over
        // consecutive destinations), else applied here (tiles of many low
        // in-degree destinations, and the spanning ones)
        TileGeo<EPL> tg;
        auto apply = [&](uint32_t k, unsigned long long val, int kind) {
            if (kind != EMIT_COMPLETE && s.shead) {
                // a spanning destination: sssp_split_kernel writes and counts it
                // after this launch; the 32-bit copy and the hub cache take the
                // tile's minimum now, so that later tiles gather it
                (kind == EMIT_HEAD ? s.shead : s.stail)[t] = val;
                if (val != NONE64) {
                    const uint32_t vtx = g.dst_ident ? k : g.dst_id[k];
                    dist32_put(s, vtx, val, false);
                    hub_min(vtx, val);
                }
                return;
            }
            if (val == NONE64)
                return;
            const uint32_t vtx = g.dst_ident ? k : g.dst_id[k];
            if (kind == EMIT_COMPLETE) { /* the destination's only writer in this launch */
                if (val < cur_dist(vtx)) {
                    s.prop64[vtx] = val;
                    dist32_put(s, vtx, val, true);
                    hub_min(vtx, val);
                    activate_new(vtx);
                }
            } else if (val < s.prop64[vtx] && val < atomicMin(&s.prop64[vtx], val)) {
                dist32_put(s, vtx, val, false);
                hub_min(vtx, val);
                activate(vtx);
            }
        };
        if constexpr (SUMS32) {
            uint32_t v[EPL];
#pragma unroll
            for (int q = 0; q < EPL; ++q) {
                const uint32_t x = sa[q];
                bool on = x != NONE32;
                if (filtered && on)
                    on = (ld_ro_u32(cur + (x >> 5)) >> (x & 31u)) & 1u; /* changed by the previous pull */
                // global memory only for sources past the hub cache, behind a
                // branch (measured 7% faster per dense pull than a select of
                // the two loads)
                uint32_t gy = NONE32;
                if (on && x >= hub_lim)
                    gy = ld_gather_u32(s.dist32 + x);
                const uint32_t y = on ? ((x < hub_lim) ? hub32[x] : gy) : NONE32;
                const uint32_t w = (wword[q >> 2] >> (8 * (q & 3))) & 0xFFu;
                uint32_t sum = y + w; /* phase_edge_pull_sssp.c:136-137 */
                if (y != NONE32 && (sum < y || sum >= lim)) {
                    dropped = true;
                    sum = NONE32;
                }
                v[q] = (y == NONE32) ? NONE32 : sum;
            }
            tile_geometry_bits<EPL>(g, base, t + 1u >= T, k0, kend, lane, tg);
            seg_reduce<EPL>(v, tg, lane, MinU32(), [&](uint32_t k, uint32_t val, int kind) {
                const uint32_t slot = k - tg.k0;
                if (kind == EMIT_COMPLETE && slot < SLOTS)
                    my_min32[slot] = val;
                else
                    apply(k, val == NONE32 ? NONE64 : (unsigned long long)val, kind);
            });
        } else {
            unsigned long long v[EPL];
#pragma unroll
            for (int q = 0; q < EPL; ++q) {
                const uint32_t x = sa[q];
                bool on = x != NONE32;
                if (filtered && on)
                    on = (ld_ro_u32(cur + (x >> 5)) >> (x & 31u)) & 1u; /* changed by the previous pull */
                unsigned long long d = NONE64;
                if (on && narrow) {
                    const uint32_t y = (x < hub_lim) ? hub32[x] : ld_gather_u32(s.dist32 + x);
                    d = (y == NONE32) ? NONE64 : (unsigned long long)y;
                } else if (on) {
                    d = (x < hub_lim) ? hub64[x] : s.prop64[x];
                }
                const unsigned long long w = (wword[q >> 2] >> (8 * (q & 3))) & 0xFFu;
                v[q] = (d == NONE64) ? NONE64 : d + w; /* phase_edge_pull_sssp.c:136-137 */
            }
            tile_geometry_bits<EPL>(g, base, t + 1u >= T, k0, kend, lane, tg);
            seg_reduce<EPL>(v, tg, lane, MinU64(), [&](uint32_t k, unsigned long long val, int kind) {
                const uint32_t slot = k - tg.k0;
                if (kind == EMIT_COMPLETE && slot < SLOTS)
                    my_min64[slot] = val;
                else
                    apply(k, val, kind);
            });
        }
        dsts += tg.ndst;
        __syncwarp();
        const uint32_t nd = tg.ndst;
        const uint32_t jlo = tg.k0_fresh ? 0u : 1u;
        const uint32_t jhi = min(tg.tail_cont ? nd - 1u : nd, SLOTS);
        // the staged complete destinations, 32 consecutive ones per round; each
        // is this launch's only writer of its vertex, so its frontier bit is
        // new: the bits of a round go out as one atomicOr per distinct word
        for (uint32_t j0 = 0; j0 < jhi; j0 += 32u) { /* warp-uniform rounds */
            const uint32_t j = j0 + (uint32_t)lane;
            unsigned long long val = NONE64;
            if (j >= jlo && j < jhi) {
                if constexpr (SUMS32) {
                    const uint32_t x = my_min32[j];
                    val = x == NONE32 ? NONE64 : (unsigned long long)x;
                } else {
                    val = my_min64[j];
                }
            }
            bool chg = false;
            uint32_t vtx = 0u, od = 0u;
            if (val != NONE64) {
                vtx = g.dst_ident ? tg.k0 + j : g.dst_id[tg.k0 + j];
                if (val < cur_dist(vtx)) {
                    chg = true;
                    s.prop64[vtx] = val;
                    dist32_put(s, vtx, val, true);
                    hub_min(vtx, val);
                    od = g.outdeg[vtx];
                }
            }
            const uint32_t word = chg ? vtx >> 5 : NONE32;
            const uint32_t grp = __match_any_sync(FULL, word);
            const uint32_t bits = __reduce_or_sync(grp, chg ? 1u << (vtx & 31u) : 0u);
            if (chg && (uint32_t)lane == (uint32_t)(__ffs(grp) - 1)) {
                atomicOr(&nxt[word], bits);
                ++occ; /* a distinct word of these 32 destinations */
            }
            if (chg) {
                mass += od;
                ++act;
                count_deg(od);
            }
        }
        __syncwarp(); /* my_min is rewritten by the next tile */
    }
    if (use_hub && threadIdx.x == 0 && !mbar_wait_bounded(&hub_bar, 0u, HUB_WAIT_TRIES)) {
        atomicOr(&c->error, ERR_HUB_TIMEOUT);
        mbar_wait_bounded(&hub_bar, 0u, HUB_WAIT_TRIES);
    }
    if (__any_sync(FULL, dropped) && lane == 0) {
        atomicOr(&c->narrow_ovf, 1u);
        atomicOr(&c->ovf_redo, 1u);
    }
    {
        const unsigned long long d0 = warp_sum_u64(degs & 0x1FFFFFull);
        const unsigned long long d1 = warp_sum_u64((degs >> 21) & 0x1FFFFFull);
        const unsigned long long d2 = warp_sum_u64(degs >> 42);
        if (lane == 0) {
            atomicAdd(&sh_deg[0], (unsigned int)d0);
            atomicAdd(&sh_deg[1], (unsigned int)d1);
            atomicAdd(&sh_deg[2], (unsigned int)d2);
        }
    }
    mass = warp_sum_u64(mass);
    edges = warp_sum_u64(edges);
    act = warp_sum_u64(act);
    occ = warp_sum_u64(occ);
    if (lane == 0) {
        sh_cnt[wib][CNT_MASS] = mass;
        sh_cnt[wib][CNT_EDGES] = edges;
        sh_cnt[wib][CNT_TILES] = tiles;
        sh_cnt[wib][CNT_DSTS] = dsts;
        sh_cnt[wib][CNT_ACT] = act;
        sh_cnt[wib][CNT_OCC] = occ;
    }
    __syncthreads();
    if (threadIdx.x < NCNT) {
        unsigned long long a = 0;
        if (threadIdx.x >= CNT_DEG0 && threadIdx.x <= CNT_DEG2)
            a = sh_deg[threadIdx.x - CNT_DEG0];
        else
            for (int w = 0; w < WARPS; ++w)
                a += sh_cnt[w][threadIdx.x];
        block_cnt[NCNT * blockIdx.x + threadIdx.x] = a;
    }
}

// Destinations spanning the 512-edge SSSP pull's tiles: the minimum of their
// tiles' partials (stail of every tile but the last, shead of the last),
// compared with the 64-bit distance and written once -- this launch is their
// only writer of it (the pull lowered only the 32-bit copy), so their
// frontier bits are new.  Launched after each of the pull's two launches, for
// the destinations whose last tile that launch covered, so that the hub
// destinations' new distances reach the second launch's hub cache.  A thread
// per destination of at most SPLIT_SERIAL+1 tiles, a warp per longer one.  Its
// counters are added to the pull launch's block counters (nblk blocks).
__global__ void sssp_split_kernel(DevGraph g, DevState s, unsigned long long* block_cnt, uint32_t nblk, uint32_t phase)
{
    Ctrl* c = s.ctrl;
    if (c->done || c->mode == MODE_WEDGE)
        return;
    const uint32_t T = (uint32_t)((g.E + SSSP_TILE - 1) / SSSP_TILE);
    const uint32_t split = min(s.hub_tile, T);
    uint32_t* nxt = next_front(s, c->parity);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthr = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    unsigned long long mass = 0, act = 0, occ = 0, degs = 0;
    auto mine = [&](uint32_t t1) { return (t1 < split) == (phase == PHASE_HUBS); };
    auto apply = [&](uint32_t k, unsigned long long m) {
        if (m == NONE64)
            return;
        const uint32_t vtx = g.dst_ident ? k : g.dst_id[k];
        /* the 64-bit distance: the pull lowered the 32-bit copy already */
        if (m < s.prop64[vtx]) {
            s.prop64[vtx] = m;
            dist32_put(s, vtx, m, true);
            atomicOr(&nxt[vtx >> 5], 1u << (vtx & 31u));
            ++occ;
            const uint32_t od = g.outdeg[vtx];
            mass += od;
            ++act;
            const uint32_t bk = degree_bucket(od);
            if (bk < 3u)
                degs += 1ull << (21u * bk);
        }
    };
    for (uint32_t i = tid; i < s.pnsplit; i += nthr) {
        const uint32_t t0 = s.psplit_t0[i], t1 = s.psplit_t1[i];
        if (!mine(t1))
            continue;
        unsigned long long m = s.shead[t1];
        for (uint32_t tt = t0; tt < t1; ++tt)
            m = min(m, s.stail[tt]);
        apply(s.psplit_k[i], m);
    }
    for (uint32_t j = tid >> 5; j < s.pnwide; j += nthr >> 5) {
        const uint32_t i = s.pT - 1u - j;
        const uint32_t a = s.psplit_t0[i], b = s.psplit_t1[i];
        if (!mine(b))
            continue; /* warp-uniform */
        unsigned long long m = NONE64;
        for (uint32_t tt = a + (uint32_t)lane; tt < b; tt += 32u)
            m = min(m, s.stail[tt]);
#pragma unroll
        for (int d = 16; d > 0; d >>= 1)
            m = min(m, __shfl_xor_sync(FULL, m, d));
        if (lane == 0)
            apply(s.psplit_k[i], min(m, s.shead[b]));
    }
    mass = warp_sum_u64(mass);
    act = warp_sum_u64(act);
    occ = warp_sum_u64(occ);
    const unsigned long long d0 = warp_sum_u64(degs & 0x1FFFFFull);
    const unsigned long long d1 = warp_sum_u64((degs >> 21) & 0x1FFFFFull);
    const unsigned long long d2 = warp_sum_u64(degs >> 42);
    if (lane == 0 && (mass | act | occ)) {
        unsigned long long* bc = block_cnt + (uint64_t)NCNT * (((uint64_t)blockIdx.x * (AUX_THREADS / 32) + (threadIdx.x >> 5)) % nblk);
        atomicAdd(&bc[CNT_MASS], mass);
        atomicAdd(&bc[CNT_ACT], act);
        atomicAdd(&bc[CNT_OCC], occ);
        atomicAdd(&bc[CNT_DEG0], d0);
        atomicAdd(&bc[CNT_DEG1], d1);
        atomicAdd(&bc[CNT_DEG2], d2);
    }
}

// The per-destination work of a dense pull, one destination per lane, launched
// before the tile pull (pull_kernel): the BFS probe; the CC probe; CC's first
// pull over engine-id labels (launch A: the hub destinations, launch B: the
// rest).  Latency-bound chains of a few dependent loads: 32 registers, two
// 1024-thread blocks per SM, so twice the warps of the tile pull are in
// flight.  block_cnt as pull_kernel's.
template <int APP, int EPL>
__global__ void __launch_bounds__(PULL_THREADS, 2)
    dst_kernel(DevGraph g, DevState s, unsigned long long* block_cnt, uint32_t phase)
{
    constexpr int WARPS = PULL_THREADS / 32;
    constexpr uint32_t TILE_E = 32u * EPL;
    __shared__ unsigned long long sh_cnt[WARPS][NCNT];
    __shared__ unsigned int sh_deg[3];
    Ctrl* c = s.ctrl;
    if (c->done)
        return;
    const uint32_t mode = c->mode;
    // CC on a symmetric graph propagates engine ids; before its first pull every
    // label is its vertex's own id
    const bool ident0 = APP == WEDGE_APP_CC && g.sym != 0u && c->iter == 0u;
    const bool cand = (APP == WEDGE_APP_BFS || APP == WEDGE_APP_CC) && mode == MODE_WEDGE && s.cand != nullptr;
    if ((mode != MODE_DENSE && !cand) || (phase == PHASE_DST_B && !ident0)) {
        // nothing to do before this pull: report zeros
        if (threadIdx.x < NCNT)
            block_cnt[NCNT * blockIdx.x + threadIdx.x] = 0ull;
        return;
    }
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t* cur = cur_front(s, c->parity);
    uint32_t* nxt = next_front(s, c->parity);
    const unsigned long long pwin = c->probe_edges; /* probe window of this pull */
    unsigned long long mass = 0, edges = 0, dsts = 0, act = 0, occ = 0;
    if (threadIdx.x < 3)
        sh_deg[threadIdx.x] = 0u;
    __syncthreads();
    // Bits into the pull's output bitmap, and the count of its words they
    // occupy (no atomic returns: a word only this warp writes in the launch
    // counts once; lanes' scattered bits count once per distinct word of the
    // warp's group, count_words after the group)
    auto set_word = [&](uint32_t w, uint32_t bits) {
        atomicOr(&nxt[w], bits);
        ++occ;
    };
    auto count_words = [&](uint32_t dw) {
        const uint32_t same = __match_any_sync(FULL, dw);
        if (dw != NONE32 && (uint32_t)(__ffs(same) - 1) == (uint32_t)lane)
            ++occ;
    };

    // bitmap marks of tiles [ta, tb] (one lane)
    auto mark_tiles = [](uint32_t* bm, uint32_t ta, uint32_t tb) {
        for (uint32_t w = ta >> 5; w <= (tb >> 5); ++w) {
            const uint32_t a = (w == (ta >> 5)) ? (ta & 31u) : 0u;
            const uint32_t z = (w == (tb >> 5)) ? (tb & 31u) : 31u;
            atomicOr(&bm[w], (z == 31u ? FULL : ((2u << z) - 1u)) & ~((1u << a) - 1u));
        }
    };
    // tiles [ta, tb] into the tile pull's work: the lane that sets a tile's
    // tile_need bit appends the tile to tile_list, so each is listed once
    auto need_tiles = [&](uint32_t ta, uint32_t tb) {
        for (uint32_t w = ta >> 5; w <= (tb >> 5); ++w) {
            const uint32_t a = (w == (ta >> 5)) ? (ta & 31u) : 0u;
            const uint32_t z = (w == (tb >> 5)) ? (tb & 31u) : 31u;
            const uint32_t m = (z == 31u ? FULL : ((2u << z) - 1u)) & ~((1u << a) - 1u);
            uint32_t fresh = m & ~atomicOr(&s.tile_need[w], m);
            if (fresh) {
                uint32_t pos = atomicAdd(&c->need_n, (uint32_t)__popc(fresh));
                for (; fresh; fresh &= fresh - 1u)
                    s.tile_list[pos++] = (unsigned long long)(w * 32u + (uint32_t)(__ffs(fresh) - 1)) << 32;
            }
        }
    };
    // Open-tile marks of the warp's destinations left unfinished (tiles [ta, tb],
    // none where ta > tb; the bitmap is rebuilt by every dense pull).  The lanes'
    // destinations are consecutive, so most of their tiles share a word: one
    // atomic per distinct word.  Called by all lanes.
    auto mark_open = [&](uint32_t ta, uint32_t tb) {
        const bool one = ta <= tb && (ta >> 5) == (tb >> 5);
        if (ta <= tb && !one)
            mark_tiles(s.tile_open, ta, tb);
        const uint32_t bits = one ? ((tb & 31u) == 31u ? FULL : ((2u << (tb & 31u)) - 1u)) & ~((1u << (ta & 31u)) - 1u) : 0u;
        uint32_t pending = __ballot_sync(FULL, one);
        while (pending) {
            const int leader = __ffs(pending) - 1;
            const uint32_t w = __shfl_sync(FULL, ta >> 5, leader);
            const bool mine = one && (ta >> 5) == w;
            const uint32_t all = __reduce_or_sync(FULL, mine ? bits : 0u);
            if (lane == leader)
                atomicOr(&s.tile_open[w], all);
            pending &= ~__ballot_sync(FULL, mine);
        }
    };

    if (APP == WEDGE_APP_CC && ident0) {
        // The first CC pull over engine-id labels, one destination per lane.  A
        // source outside the hub range [0, hub_n) still holds its own id, and a
        // destination's sources ascend, so past its hub sources only the first
        // one can lower the minimum; the hub sources' labels are final once the
        // hub launch (the destinations with ids < hub_n) is over.  The hub launch
        // itself sees every label at its id: the first source decides.  This is
        // the tile pull's result for the same labels without reading the other
        // in-edges (Jacobi for the hubs, where the tile pull lets a block's
        // warps see each other's hub updates).
        const bool hubs = phase == PHASE_DST_A;
        const uint32_t kb = hubs ? 0u : s.hub_k, ke = hubs ? s.hub_k : g.Vne;
        const uint32_t hn = s.hub_n;
        const uint32_t nthr = gridDim.x * blockDim.x;
        // the next group's offsets are loaded while this one is processed
        unsigned long long plo = 0ull, phi = 0ull;
        auto prefetch = [&](uint32_t b) {
            const uint32_t kk = b + (uint32_t)lane;
            if (kk < ke) {
                plo = g.dst_off[kk];
                phi = g.dst_off[kk + 1u];
            }
        };
        prefetch(kb + gw * 32u);
        for (uint32_t base = kb + gw * 32u; base < ke; base += nthr) {
            const uint32_t k = base + (uint32_t)lane;
            const unsigned long long lo = plo, hi = phi;
            prefetch(base + nthr);
            bool chg = false, zero = false;
            uint32_t d = 0u, od = 0u;
            if (k < ke) {
                d = g.dst_ident ? k : g.dst_id[k];
                uint32_t m = d;
                unsigned long long e = lo;
                while (e < hi) {
                    const uint32_t x = g.src[e++];
                    if (hubs || x >= hn) {
                        m = x < m ? x : m;
                        break;
                    }
                    const uint32_t l = s.prop32[x];
                    m = l < m ? l : m;
                    if (m == 0u)
                        break;
                }
                edges += e - lo;
                chg = m < d;
                zero = chg && m == 0u;
                if (chg) {
                    s.prop32[d] = m; /* the destination's only writer */
                    od = g.outdeg[d];
                    mass += od;
                    ++act;
                }
            }
            dsts += (uint64_t)__popc(__ballot_sync(FULL, k < ke));
#pragma unroll
            for (uint32_t b = 0; b < 3u; ++b) {
                const uint32_t nb = __popc(__ballot_sync(FULL, chg && degree_bucket(od) == b));
                if (lane == 0 && nb)
                    atomicAdd(&sh_deg[b], nb);
            }
            if (g.dst_ident) { /* d = k: the lanes' bits fall in two words at most */
                const uint32_t w0 = base >> 5;
                const bool in0 = (k >> 5) == w0;
                const uint32_t bit = 1u << (k & 31u);
                const uint32_t c0 = __reduce_or_sync(FULL, (chg && in0) ? bit : 0u);
                const uint32_t c1 = __reduce_or_sync(FULL, (chg && !in0) ? bit : 0u);
                const uint32_t z0 = __reduce_or_sync(FULL, (zero && in0) ? bit : 0u);
                const uint32_t z1 = __reduce_or_sync(FULL, (zero && !in0) ? bit : 0u);
                if (lane == 0) {
                    if (c0)
                        set_word(w0, c0);
                    if (c1)
                        set_word(w0 + 1u, c1);
                    if (z0)
                        atomicOr(&s.vis_c[w0], z0); /* label 0 is final */
                    if (z1)
                        atomicOr(&s.vis_c[w0 + 1u], z1);
                }
            } else {
                if (chg)
                    atomicOr(&nxt[d >> 5], 1u << (d & 31u));
                if (zero)
                    atomicOr(&s.vis_c[k >> 5], 1u << (k & 31u));
                count_words(chg ? d >> 5 : NONE32);
            }
        }
    }
    if (APP == WEDGE_APP_BFS && cand) {
        // A Wedge pull over the candidates the last build listed (unvisited
        // destinations with an in-edge from the frontier): the probe below for
        // each, one per lane, in list order.  The lanes clear the candidates'
        // bitmap words for the next build (every bit set there is in the list).
        const uint32_t n = c->cand_n;
        const uint32_t nthr = gridDim.x * blockDim.x;
        for (uint32_t base = gw * 32u; base < n; base += nthr) {
            const uint32_t i = base + (uint32_t)lane;
            bool hit = false;
            uint32_t od = 0u, dw = NONE32;
            if (i < n) {
                const uint32_t k = s.cand_list[i];
                s.cand[k >> 5] = 0u;
                const uint32_t d = g.dst_ident ? k : g.dst_id[k];
                const unsigned long long lo = g.dst_off[k], hi = g.dst_off[k + 1u];
                const unsigned long long lim = hi - lo > pwin ? lo + pwin : hi;
                unsigned long long e = lo;
                uint32_t par = NONE32;
                while (e < lim) {
                    const uint32_t x = g.src[e++];
                    if ((ld_ro_u32(cur + (x >> 5)) >> (x & 31u)) & 1u) {
                        par = x;
                        break;
                    }
                }
                edges += e - lo;
                hit = par != NONE32;
                if (!hit && lim < hi)
                    need_tiles((uint32_t)(lim / TILE_E), (uint32_t)((hi - 1u) / TILE_E));
                if (hit) {
                    s.prop32[d] = par; /* the destination's only writer in this launch */
                    atomicOr(&s.vis_c[k >> 5], 1u << (k & 31u));
                    atomicOr(&nxt[d >> 5], 1u << (d & 31u));
                    dw = d >> 5;
                    od = g.outdeg[d];
                    mass += od;
                    ++act;
                }
            }
            count_words(dw);
            dsts += (uint64_t)__popc(__ballot_sync(FULL, i < n));
#pragma unroll
            for (uint32_t b = 0; b < 3u; ++b) {
                const uint32_t nb = __popc(__ballot_sync(FULL, hit && degree_bucket(od) == b));
                if (lane == 0 && nb)
                    atomicAdd(&sh_deg[b], nb);
            }
        }
    } else if (APP == WEDGE_APP_BFS) {
        // Bottom-up probe, one unvisited destination per lane: its first
        // PROBE_EDGES sources in ascending order, up to the first one in the
        // frontier -- the least frontier source, the value the tile pull's min
        // would give it.  A destination whose sources it read to the end
        // without a hit has no parent this iteration (the frontier is fixed
        // during a pull); one with sources left marks the tiles holding them in
        // tile_need, the only tiles the tile pull (the next launch) walks.
        const uint32_t nthr = gridDim.x * blockDim.x;
        // the next group's visited word and offsets are loaded while this one is
        // probed (each group's vis_c word belongs to its warp alone)
        uint32_t pv = 0u;
        unsigned long long plo = 0ull, phi = 0ull;
        auto prefetch = [&](uint32_t b) {
            const uint32_t kk = b + (uint32_t)lane;
            if (b < g.Vne)
                pv = s.vis_c[b >> 5];
            if (kk < g.Vne) {
                plo = g.dst_off[kk];
                phi = g.dst_off[kk + 1u];
            }
        };
        prefetch(gw * 32u);
        for (uint32_t base = gw * 32u; base < g.Vne; base += nthr) {
            const uint32_t k = base + (uint32_t)lane; /* base is a multiple of 32: one vis_c word */
            const uint32_t vw = pv;
            const unsigned long long lo = plo, hi = phi;
            prefetch(base + nthr);
            const bool todo = k < g.Vne && !((vw >> lane) & 1u);
            bool hit = false;
            uint32_t od = 0u, dw = NONE32;
            uint32_t ta = 1u, tb = 0u; /* tiles of a destination left unvisited (none: ta > tb) */
            if (todo) {
                const uint32_t d = g.dst_ident ? k : g.dst_id[k];
                const unsigned long long lim = hi - lo > pwin ? lo + pwin : hi;
                unsigned long long e = lo;
                uint32_t par = NONE32;
                while (e < lim) {
                    const uint32_t x = g.src[e++];
                    if ((ld_ro_u32(cur + (x >> 5)) >> (x & 31u)) & 1u) {
                        par = x;
                        break;
                    }
                }
                edges += e - lo;
                hit = par != NONE32;
                if (!hit) {
                    ta = (uint32_t)(lo / TILE_E);
                    tb = (uint32_t)((hi - 1u) / TILE_E);
                    // sources past the window remain: the tile pull reads the tiles holding them
                    if (lim < hi)
                        need_tiles((uint32_t)(lim / TILE_E), tb);
                }
                if (hit) {
                    s.prop32[d] = par; /* the destination's only writer in this launch */
                    od = g.outdeg[d];
                    mass += od;
                    ++act;
                    if (!g.dst_ident) {
                        atomicOr(&nxt[d >> 5], 1u << (d & 31u));
                        dw = d >> 5;
                    }
                }
            }
            mark_open(ta, tb);
            count_words(dw);
            dsts += (uint64_t)__popc(__ballot_sync(FULL, todo));
#pragma unroll
            for (uint32_t b = 0; b < 3u; ++b) {
                const uint32_t nb = __popc(__ballot_sync(FULL, hit && degree_bucket(od) == b));
                if (lane == 0 && nb)
                    atomicAdd(&sh_deg[b], nb);
            }
            const uint32_t hits = __ballot_sync(FULL, hit);
            if (lane == 0 && hits) {
                atomicOr(&s.vis_c[base >> 5], hits);
                if (g.dst_ident)
                    set_word(base >> 5, hits); /* d = k */
            }
        }
    }
    if (APP == WEDGE_APP_CC && cand && phase == PHASE_DST_A) {
        // A Wedge pull over the candidates the last build listed (unfinished
        // destinations with an in-edge from a vertex the last pull changed): the
        // CC probe below for each, one per lane, in list order; the lanes clear
        // the candidates' bitmap words for the next build.
        const uint32_t n = c->cand_n;
        const uint32_t nthr = gridDim.x * blockDim.x;
        for (uint32_t base = gw * 32u; base < n; base += nthr) {
            const uint32_t i = base + (uint32_t)lane;
            bool chg = false;
            uint32_t od = 0u, dw = NONE32;
            if (i < n) {
                const uint32_t k = s.cand_list[i];
                s.cand[k >> 5] = 0u;
                const uint32_t d = g.dst_ident ? k : g.dst_id[k];
                const unsigned long long lo = g.dst_off[k], hi = g.dst_off[k + 1u];
                const unsigned long long lim = hi - lo > pwin ? lo + pwin : hi;
                const uint32_t cv = s.prop32[d];
                uint32_t m = cv;
                unsigned long long e = lo;
                while (e < lim) {
                    const uint32_t l = s.prop32[g.src[e++]];
                    m = l < m ? l : m;
                    if (m == 0u)
                        break;
                }
                edges += e - lo;
                const bool whole = m == 0u || e == hi;
                if (whole && m < cv) {
                    s.prop32[d] = m; /* the destination's only writer in this launch */
                    chg = true;
                    if (m == 0u)
                        atomicOr(&s.vis_c[k >> 5], 1u << (k & 31u)); /* label 0 is final */
                    atomicOr(&nxt[d >> 5], 1u << (d & 31u));
                    dw = d >> 5;
                    od = g.outdeg[d];
                    mass += od;
                    ++act;
                }
                if (!whole)
                    need_tiles((uint32_t)(lo / TILE_E), (uint32_t)((hi - 1u) / TILE_E));
            }
            count_words(dw);
            dsts += (uint64_t)__popc(__ballot_sync(FULL, i < n));
#pragma unroll
            for (uint32_t b = 0; b < 3u; ++b) {
                const uint32_t nb = __popc(__ballot_sync(FULL, chg && degree_bucket(od) == b));
                if (lane == 0 && nb)
                    atomicAdd(&sh_deg[b], nb);
            }
        }
    } else if (APP == WEDGE_APP_CC && !ident0 && !cand) {
        // CC probe (dense pulls after the first), one unfinished destination
        // (label not 0) per lane: the labels of its first PROBE_EDGES sources,
        // hubs first, up to the first label 0, the least label there is.  Where
        // that found 0 or read every source, the minimum is the whole pull's for
        // the labels read and is applied here; a longer destination without a 0
        // marks its tiles for the tile pull (the next two launches), which walks
        // only those.
        const uint32_t nthr = gridDim.x * blockDim.x;
        // the next group's finished word and offsets are loaded while this one
        // is probed (each group's vis_c word belongs to its warp alone)
        uint32_t pv = 0u;
        unsigned long long plo = 0ull, phi = 0ull;
        auto prefetch = [&](uint32_t b) {
            const uint32_t kk = b + (uint32_t)lane;
            if (b < g.Vne)
                pv = s.vis_c[b >> 5];
            if (kk < g.Vne) {
                plo = g.dst_off[kk];
                phi = g.dst_off[kk + 1u];
            }
        };
        prefetch(gw * 32u);
        for (uint32_t base = gw * 32u; base < g.Vne; base += nthr) {
            const uint32_t k = base + (uint32_t)lane; /* base is a multiple of 32: one vis_c word */
            const uint32_t vw = pv;
            const unsigned long long lo = plo, hi = phi;
            prefetch(base + nthr);
            const bool todo = k < g.Vne && !((vw >> lane) & 1u);
            bool chg = false, zero = false;
            uint32_t dw = NONE32;
            uint32_t d = 0u, od = 0u;
            uint32_t ta = 1u, tb = 0u;
            if (todo) {
                d = g.dst_ident ? k : g.dst_id[k];
                const unsigned long long lim = hi - lo > pwin ? lo + pwin : hi;
                const uint32_t cv = s.prop32[d];
                uint32_t m = cv;
                unsigned long long e = lo;
                while (e < lim) {
                    const uint32_t l = s.prop32[g.src[e++]];
                    m = l < m ? l : m;
                    if (m == 0u)
                        break;
                }
                edges += e - lo;
                const bool whole = m == 0u || e == hi;
                if (whole && m < cv) {
                    s.prop32[d] = m; /* the destination's only writer in this launch */
                    chg = true;
                    zero = m == 0u;
                    od = g.outdeg[d];
                    mass += od;
                    ++act;
                    if (!g.dst_ident) {
                        atomicOr(&nxt[d >> 5], 1u << (d & 31u));
                        dw = d >> 5;
                    }
                }
                if (!whole)
                    need_tiles((uint32_t)(lo / TILE_E), (uint32_t)((hi - 1u) / TILE_E));
                if (!zero) {
                    ta = (uint32_t)(lo / TILE_E);
                    tb = (uint32_t)((hi - 1u) / TILE_E);
                }
            }
            mark_open(ta, tb);
            count_words(dw);
            dsts += (uint64_t)__popc(__ballot_sync(FULL, todo));
#pragma unroll
            for (uint32_t b = 0; b < 3u; ++b) {
                const uint32_t nb = __popc(__ballot_sync(FULL, chg && degree_bucket(od) == b));
                if (lane == 0 && nb)
                    atomicAdd(&sh_deg[b], nb);
            }
            const uint32_t chgs = __ballot_sync(FULL, chg), zeros = __ballot_sync(FULL, zero);
            if (lane == 0) {
                if (zeros)
                    atomicOr(&s.vis_c[base >> 5], zeros); /* label 0 is final */
                if (chgs && g.dst_ident)
                    set_word(base >> 5, chgs); /* d = k */
            }
        }
    }
    mass = warp_sum_u64(mass);
    edges = warp_sum_u64(edges);
    act = warp_sum_u64(act);
    occ = warp_sum_u64(occ);
    if (lane == 0) {
        sh_cnt[wib][CNT_MASS] = mass;
        sh_cnt[wib][CNT_EDGES] = edges;
        sh_cnt[wib][CNT_TILES] = 0ull;
        sh_cnt[wib][CNT_DSTS] = dsts; // warp-uniform
        sh_cnt[wib][CNT_ACT] = act;
        sh_cnt[wib][CNT_DEG0] = 0ull;
        sh_cnt[wib][CNT_DEG1] = 0ull;
        sh_cnt[wib][CNT_DEG2] = 0ull;
        sh_cnt[wib][CNT_OCC] = occ;
    }
    __syncthreads();
    if (threadIdx.x < NCNT) {
        unsigned long long a = 0;
        for (int w = 0; w < WARPS; ++w)
            a += sh_cnt[w][threadIdx.x];
        if (threadIdx.x >= CNT_DEG0 && threadIdx.x <= CNT_DEG2)
            a = sh_deg[threadIdx.x - CNT_DEG0];
        block_cnt[NCNT * blockIdx.x + threadIdx.x] = a;
    }
}

// the fixed schedules; WEDGE_SCHED_LEARNED and WEDGE_SCHED_PROBE fall back to
// the plain rule here (decide_kernel overrides it where they apply)
__device__ __forceinline__ uint32_t choose_mode(uint32_t sched, unsigned long long mass, unsigned long long thr)
{
    if (sched == WEDGE_SCHED_DENSE)
        return MODE_DENSE;
    if (sched == WEDGE_SCHED_WEDGE)
        return MODE_WEDGE;
    if (sched == WEDGE_SCHED_FILTERED)
        return MODE_FILTERED;
    return mass > thr ? MODE_DENSE : MODE_WEDGE; /* execution_bfs.c:141 */
}

// Scheduler features of the next iteration, from the pull just finished (its
// reduced counters) and the traversal so far.  Every feature is O(1) in size.
// Single-precision arithmetic: one thread computes them after every pull, and
// the FP64 units of this GPU are slow.
__device__ void sched_features(const DevGraph& g, const Ctrl* c, uint32_t app, const unsigned long long (&cnt)[NCNT],
                               float* f)
{
    const float V = (float)(g.V ? g.V : 1), E = (float)(g.E ? g.E : 1);
    const float m = (float)cnt[CNT_MASS], act = (float)cnt[CNT_ACT];
    const float a = act > 0.0f ? act : 1.0f;
    const float b0 = (float)cnt[CNT_DEG0], b1 = (float)cnt[CNT_DEG1], b2 = (float)cnt[CNT_DEG2];
    f[0] = log2f(1.0f + m) / 32.0f;         // out-edge mass of the activated vertices
    f[1] = m / E;
    f[2] = log2f(1.0f + act) / 32.0f;       // activated vertices
    f[3] = act / V;                         // frontier bitmap density
    // clustering of the changed bitmap: writes of distinct 32-vertex words
    // (per warp group) against activated vertices; 1/2 when every activated
    // vertex sits in a word of its own, near 0 when they fill whole words
    const float occ = (float)cnt[CNT_OCC];
    f[4] = occ > 0.0f ? occ / (occ + act) : 0.0f;
    f[5] = b0 / a;                          // out-degree histogram of the activated vertices
    f[6] = b1 / a;
    f[7] = b2 / a;
    f[8] = (act - b0 - b1 - b2) / a;
    f[9] = (float)c->activated / V;         // activated so far (BFS: visited fraction)
    f[10] = log2f(1.0f + (float)c->iter) / 8.0f;
    f[11] = log2f(E) / 40.0f;
    f[12] = app == WEDGE_APP_BFS ? 1.0f : 0.0f;
    f[13] = app == WEDGE_APP_CC ? 1.0f : 0.0f;
    f[14] = app == WEDGE_APP_SSSP ? 1.0f : 0.0f;
    f[15] = log2f(E / V) / 8.0f;            // average degree
}

// After a pull: reduce the block counters, count the iteration, stop when no
// edge was activated (execution_bfs.c:239-251) or at the cap, choose the next
// pull (execution_bfs.c:141, execution_cc.c:103).
__device__ __forceinline__ void reduce_counters(const unsigned long long* block_cnt, uint32_t nblocks,
                                                unsigned long long (&out)[NCNT])
{
    __shared__ unsigned long long sh[NCNT][AUX_THREADS / 32];
    unsigned long long x[NCNT];
#pragma unroll
    for (int j = 0; j < (int)NCNT; ++j)
        x[j] = 0ull;
    for (uint32_t i = threadIdx.x; i < nblocks; i += blockDim.x)
#pragma unroll
        for (int j = 0; j < (int)NCNT; ++j)
            x[j] += block_cnt[NCNT * i + j];
#pragma unroll
    for (int j = 0; j < (int)NCNT; ++j) {
        x[j] = warp_sum_u64(x[j]);
        if ((threadIdx.x & 31) == 0)
            sh[j][threadIdx.x >> 5] = x[j];
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < (int)NCNT; ++j) {
        unsigned long long t = 0;
        for (int w = 0; w < AUX_THREADS / 32; ++w)
            t += sh[j][w];
        out[j] = t;
    }
}

__device__ __forceinline__ void log_iteration(DevState& s, Ctrl* c, const unsigned long long (&cnt)[NCNT])
{
    c->edges_scanned += cnt[CNT_EDGES];
    c->tiles_scanned += cnt[CNT_TILES];
    c->dsts_scanned += cnt[CNT_DSTS];
    c->activated += cnt[CNT_ACT];
    c->pull_launches += pull_launches_of((int)s.app);
    if (c->iter < LOG_CAP) {
        IterRec& r = s.log[c->iter];
        r.mass_in = c->last_mass;
        r.mass_out = cnt[CNT_MASS];
        r.edges = cnt[CNT_EDGES];
        r.tiles = cnt[CNT_TILES];
        r.dsts = cnt[CNT_DSTS];
        r.activated = cnt[CNT_ACT];
        r.mode = c->mode;
        r.iter = c->iter;
    }
    c->iter += 1u;
}

// After a pull: reduce the block counters, count the iteration, stop when no
// edge was activated (execution_bfs.c:239-251) or at the cap, choose the next
// pull (execution_bfs.c:141, execution_cc.c:103).
__global__ void decide_kernel(DevGraph g, DevState s, const unsigned long long* block_cnt, uint32_t nblocks, uint32_t app)
{
    Ctrl* c = s.ctrl;
    if (c->done)
        return;
    const uint32_t nsum = ((g.T + TILES_PER_REGION - 1) / TILES_PER_REGION + 31) / 32;
    for (uint32_t i = threadIdx.x; i < nsum; i += blockDim.x)
        s.summary[i] = 0u; /* the pull has cleared every chunk word it walked */
    unsigned long long cnt[NCNT];
    reduce_counters(block_cnt, nblocks, cnt);
    __shared__ float feat[NF], xs[NF], h1[NH], h2[NH], pred[NO];
    __shared__ uint32_t go;
    if (threadIdx.x == 0) {
        const unsigned long long m = cnt[CNT_MASS];
        if (c->mode == MODE_WEDGE)
            c->wedge_iters += 1u;
        log_iteration(s, c, cnt);
        c->last_mass = m;
        c->mass = m;
        c->parity ^= 1u;
        c->need_n = 0u;
        c->cand_n = 0u;
        c->tiles = 0u;
        c->items = 0u;
        c->alist_n = 0u;
        go = 0u;
        // SSSP: a pull dropped 32-bit sums that reached the copy's limit; the
        // next pull is dense and 64-bit, and relaxes every in-edge again
        const bool redo = c->ovf_redo != 0u;
        c->ovf_redo = 0u;
        if (m == 0ull && !redo) {
            c->done = 1u;
            c->loop = 0u;
        } else if (c->iter >= c->max_iter) {
            c->done = 1u;
            c->not_converged = 1u;
            c->loop = 0u;
        } else {
            c->mode = choose_mode(c->sched, m, c->threshold);
            if (c->sched == WEDGE_SCHED_PROBE && c->iter == c->probe_iter)
                c->mode = c->probe_mode;
            sched_features(g, c, app, cnt, feat);
            if (c->iter < LOG_CAP) {
                for (int i = 0; i < NF; ++i)
                    s.log[c->iter].feat[i] = feat[i];
                s.log[c->iter].learned = 0u;
            }
            go = (c->sched == WEDGE_SCHED_LEARNED && s.net) ? 1u : 0u;
            if (redo) {
                c->mode = MODE_DENSE;
                go = 0u;
            }
        }
    }
    __syncthreads();
    if (!go)
        return;
    // the scheduler network: predicted log2 cost of each strategy
    sched_forward_block(s.net, feat, xs, h1, h2, pred);
    if (threadIdx.x == 0) {
        const float* net = s.net;
        bool in_range = true;
        for (int i = 0; i < NF; ++i)
            in_range = in_range && feat[i] >= net[OFF_LO + i] && feat[i] <= net[OFF_HI + i];
        uint32_t best = MODE_DENSE;
        for (uint32_t k = 1; k < (uint32_t)NO; ++k)
            if (pred[k] < pred[best])
                best = k;
        if (app == WEDGE_APP_BFS && best == MODE_FILTERED)
            best = MODE_DENSE; /* the BFS pull has no separate filtered form */
        const uint32_t plain = c->mode;
        if (in_range && best != plain && pred[plain] - pred[best] >= net[OFF_MARGIN]) {
            c->mode = best;
            c->learned_iters += 1u;
            if (c->iter < LOG_CAP)
                s.log[c->iter].learned = 1u;
        }
    }
}

// chunk of a CSRI entry (an in-edge position, or a chunk id on graphs too large for 32-bit positions)
__device__ __forceinline__ uint32_t csri_chunk(const DevGraph& g, uint32_t x) { return g.csri_pos ? x / CHUNK : x; }

// chunks per pull tile of an application, as a shift (tile = 32 * EPL in-edges)
__device__ __forceinline__ uint32_t chunk_tile_shift(uint32_t app)
{
    const uint32_t epl = app == WEDGE_APP_CC ? (uint32_t)WEDGE_EPL_CC : 8u;
    return 31u - (uint32_t)__clz(epl);
}


// Wedge build over in-edge positions (BFS, CC): the destination of in-edge
// pos, if unfinished (BFS unvisited, CC label not 0), becomes a candidate of
// the next pull, listed once (its cand bit).
// Warp-collective: every lane calls it, with valid false where it has no edge.
__device__ __forceinline__ void add_candidate(const DevGraph& g, const DevState& s, uint32_t pos, bool valid)
{
    uint32_t k = 0;
    bool add = false;
    if (valid && s.tile_open) { /* a closed tile has no unfinished destination */
        const uint32_t t = pos >> (5u + chunk_tile_shift(s.app));
        valid = (s.tile_open[t >> 5] >> (t & 31u)) & 1u;
    }
    if (valid) {
        k = dst_of_pos(g, pos);
        const uint32_t b = 1u << (k & 31u);
        if (!(s.vis_c[k >> 5] & b) && !(s.cand[k >> 5] & b))
            add = !(atomicOr(&s.cand[k >> 5], b) & b);
    }
    const uint32_t m = __ballot_sync(FULL, add);
    if (m) {
        const int lane = threadIdx.x & 31, first = __ffs(m) - 1;
        uint32_t base = 0;
        if (lane == first)
            base = atomicAdd(&s.ctrl->cand_n, (uint32_t)__popc(m));
        base = __shfl_sync(FULL, base, first);
        if (add)
            s.cand_list[base + (uint32_t)__popc(m & ((1u << lane) - 1u))] = k;
    }
}

// set the Wedge-frontier bit of chunk ch (wedge.c:22-31) and the summary bit
// of its region.  Fire-and-forget atomics behind plain-load checks: bits are
// only set while the frontier is built, so a stale read can only cost a
// redundant atomic, and no thread waits for an atomic's return.
// Chunks of closed tiles (every destination finished) are left out:
// compact_kernel would drop them from the tile list.
__device__ __forceinline__ void mark_chunk(const DevState& s, uint32_t ch, bool valid)
{
    if (!valid)
        return;
    if (s.tile_open) {
        const uint32_t t = ch >> chunk_tile_shift(s.app);
        if (!((s.tile_open[t >> 5] >> (t & 31u)) & 1u))
            return;
    }
    const uint32_t word = ch >> 5, bit = 1u << (ch & 31u);
    if (!(s.chunk_bits[word] & bit)) {
        atomicOr(&s.chunk_bits[word], bit);
        const uint32_t r = word / REGION_WORDS, rb = 1u << (r & 31u);
        if (!(s.summary[r >> 5] & rb))
            atomicOr(&s.summary[r >> 5], rb);
    }
}

// Clears the bitmap the next pull writes and, before a dense pull, the tile
// bitmaps its probe rebuilds (every thread of the grid takes part)
__device__ __forceinline__ void advance_body(const DevGraph& g, const DevState& s, const Ctrl* c)
{
    uint32_t* fb = next_front(s, c->parity);
    const uint64_t nwords = (g.V + 31) / 32;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nwords; i += (uint64_t)gridDim.x * blockDim.x)
        fb[i] = 0u;
    // a dense pull next: its probe (CC's first: its hub/rest launches) marks
    // both afresh; a candidate Wedge pull's probe marks the needed tiles
    // (CC's first pull over engine ids rebuilds nothing: the bitmap keeps
    // init's every-tile-open until the next dense probe)
    const bool dense = c->mode == MODE_DENSE && !(s.app == WEDGE_APP_CC && g.sym && c->iter == 0u);
    if (s.tile_need && (dense || s.cand)) {
        const uint64_t twords = (uint64_t)g.T / 32 + 2;
        for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < twords; i += (uint64_t)gridDim.x * blockDim.x) {
            s.tile_need[i] = 0u;
            if (dense)
                s.tile_open[i] = 0u;
        }
    }
}

// Wedge frontier generation (wedge.c:63-155), in three launches:
//   collect_kernel  the bitmap of vertices the last pull activated -> a vertex
//                   list (one warp per 32 words, one atomic per warp)
//   expand_kernel   one thread per listed vertex marks the chunk of each of its
//                   out-edges (wedge.c:37-46); lists longer than BIG_LIST go to
//                   PIECE-sized work items instead (one atomic per warp)
//   wedge_build_kernel  one warp per work item
// Threads, not warps, expand the short lists so that enough independent
// CSRI reads are in flight: the degree relabelling puts the activated
// low-degree vertices of a BFS level in long runs of dense bitmap words.
__global__ void collect_kernel(DevGraph g, DevState s, uint32_t app)
{
    Ctrl* c = s.ctrl;
    if (c->done)
        return;
    advance_body(g, s, c); /* a different bitmap from the one collected here */
    if (c->mode != MODE_WEDGE)
        return;
    const uint32_t* fb = cur_front(s, c->parity);
    const uint64_t nwords = (g.V + 31) / 32;
    const int lane = threadIdx.x & 31;
    const uint64_t gw = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5;
    const uint64_t nw = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t base = gw * 32; base < nwords; base += nw * 32) {
        const uint32_t word = (base + lane < nwords) ? fb[base + lane] : 0u;
        const uint32_t n = __popc(word);
        uint32_t incl = n;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, d);
            if (lane >= d)
                incl += y;
        }
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        if (total == 0u)
            continue;
        uint32_t pos = 0;
        if (lane == 0)
            pos = atomicAdd(&c->alist_n, total);
        pos = __shfl_sync(FULL, pos, 0) + (incl - n);
        uint32_t bits = word;
        const uint32_t v0 = (uint32_t)((base + (uint64_t)lane) * 32u);
        while (bits) {
            const int b = __ffs(bits) - 1;
            bits &= bits - 1u;
            s.alist[pos++] = v0 + (uint32_t)b;
        }
    }
}

__global__ void expand_kernel(DevGraph g, DevState s)
{
    Ctrl* c = s.ctrl;
    if (c->done || c->mode != MODE_WEDGE)
        return;
    const int lane = threadIdx.x & 31;
    const uint32_t n = c->alist_n;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    // every lane of a warp runs the same rounds (warp-wide item appends)
    for (uint64_t i0 = (blockIdx.x * (uint64_t)blockDim.x) + (threadIdx.x & ~31u); i0 < n; i0 += stride) {
        const uint64_t i = i0 + (uint64_t)lane;
        uint32_t v = 0, np = 0;
        unsigned long long start = 0, len = 0;
        if (i < n) {
            v = s.alist[i];
            start = g.csri_off[v];
            len = g.csri_off[v + 1] - start;
            if (len > BIG_LIST) {
                np = (uint32_t)((len + PIECE - 1) / PIECE);
                len = 0;
            }
            if (s.push)
                len = 0; /* SSSP over in-edge positions: the pull relaxes the short lists itself */
        }
        // a short list's entries are loaded together, then marked
        uint32_t ch[BIG_LIST];
#pragma unroll
        for (uint32_t j = 0; j < BIG_LIST; ++j)
            ch[j] = (j < len) ? g.csri[start + j] : 0u;
        if (s.cand) {
#pragma unroll
            for (uint32_t j = 0; j < BIG_LIST; ++j)
                add_candidate(g, s, ch[j], j < len);
        } else {
#pragma unroll
            for (uint32_t j = 0; j < BIG_LIST; ++j)
                mark_chunk(s, csri_chunk(g, ch[j]), j < len);
        }
        uint32_t incl = np;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, d);
            if (lane >= d)
                incl += y;
        }
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        if (total) {
            uint32_t pos = 0;
            if (lane == 0)
                pos = atomicAdd(&c->items, total);
            pos = __shfl_sync(FULL, pos, 0) + (incl - np);
            for (uint32_t q = 0; q < np; ++q)
                s.items[pos + q] = make_uint2(v, q);
        }
    }
}

__global__ void wedge_build_kernel(DevGraph g, DevState s)
{
    Ctrl* c = s.ctrl;
    if (c->done || c->mode != MODE_WEDGE || s.push) /* SSSP over in-edge positions: the pull takes the items */
        return;
    const int lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t n = c->items;
    for (uint32_t i = gw; i < n; i += nw) {
        const uint2 it = s.items[i];
        const unsigned long long lo = g.csri_off[it.x] + (unsigned long long)it.y * PIECE;
        const unsigned long long end = g.csri_off[it.x + 1];
        const unsigned long long hi = (lo + PIECE < end) ? lo + PIECE : end;
        for (unsigned long long j0 = lo; j0 < hi; j0 += 32) {
            const unsigned long long j = j0 + lane;
            const bool valid = j < hi;
            const uint32_t x = valid ? g.csri[j] : 0u;
            if (s.cand)
                add_candidate(g, s, x, valid);
            else
                mark_chunk(s, csri_chunk(g, x), valid);
        }
    }
}

// Wedge frontier -> tile list for the next pull.  Each warp takes a region of
// REGION_WORDS chunk-bitmap words, skips it when its summary bit is clear (the
// reference skips empty 256-bit frontier groups, phase_edge_pull_bfs.c:244-246),
// and appends one (tile, chunk mask) entry per tile with a marked chunk -- one
// atomic per warp -- then clears the words: the pull consumes the frontier
// (phase_edge_pull_bfs.c:256).  BFS drops tiles already closed (all visited).
template <int EPL>
__global__ void compact_kernel(DevGraph g, DevState s)
{
    constexpr uint32_t TPW = 32 / EPL;
    constexpr uint32_t MASK = (EPL >= 32) ? FULL : ((1u << EPL) - 1u);
    Ctrl* c = s.ctrl;
    if (c->done || c->mode != MODE_WEDGE || s.cand || s.push) /* over in-edge positions: no tiles */
        return;
    const int lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t nwords = (g.T + TILES_PER_WORD - 1) / TILES_PER_WORD;
    const uint32_t nregions = (nwords + REGION_WORDS - 1) / REGION_WORDS;
    for (uint32_t r = gw; r < nregions; r += nw) {
        if (!((s.summary[r >> 5] >> (r & 31u)) & 1u))
            continue;
        const uint32_t wi = r * REGION_WORDS + (uint32_t)lane;
        uint32_t word = wi < nwords ? s.chunk_bits[wi] : 0u;
        if (word && s.tile_open) {
            // tiles of this word: wi*TPW .. +TPW (TPW <= 32 of them, all in one open word)
            const uint32_t t0 = wi * TPW;
            const uint32_t open = (s.tile_open[t0 >> 5] >> (t0 & 31u)) & ((TPW >= 32) ? FULL : ((1u << TPW) - 1u));
#pragma unroll
            for (uint32_t j = 0; j < TPW; ++j)
                if (!((open >> j) & 1u))
                    word &= ~(MASK << (EPL * j));
        }
        uint32_t cnt = 0;
#pragma unroll
        for (uint32_t j = 0; j < TPW; ++j)
            cnt += ((word >> (EPL * j)) & MASK) ? 1u : 0u;
        uint32_t incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(FULL, incl, d);
            if (lane >= d)
                incl += y;
        }
        const uint32_t total = __shfl_sync(FULL, incl, 31);
        uint32_t pos = 0;
        if (lane == 31 && total)
            pos = atomicAdd(&c->tiles, total);
        pos = __shfl_sync(FULL, pos, 31) + incl - cnt;
#pragma unroll
        for (uint32_t j = 0; j < TPW; ++j) {
            const uint32_t m = (word >> (EPL * j)) & MASK;
            if (m)
                s.tile_list[pos++] = ((unsigned long long)(wi * TPW + j) << 32) | m;
        }
        if (wi < nwords)
            s.chunk_bits[wi] = 0u;
    }
}

// Clear the bitmap the next pull writes (execution_bfs.c:320-338: swap + memset;
// execution_cc.c:243-277: clear of the active bitmap).
// the iteration's last step (the phase API's WEDGE_PHASE_ADVANCE; the traversal
// loops do it inside collect_kernel)
__global__ void advance_kernel(DevGraph g, DevState s, uint32_t app)
{
    Ctrl* c = s.ctrl;
    if (c->done)
        return;
    advance_body(g, s, c);
}

// execution_initialize_{bfs,cc,sssp} bulk part; topen = BFS pull tiles
__global__ void init_kernel(DevGraph g, DevState s, uint32_t app, uint32_t topen)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    for (uint64_t v = tid; v < g.V; v += stride) {
        if (app == WEDGE_APP_BFS)
            s.prop32[v] = NONE32; /* execution_bfs.c:106 */
        else if (app == WEDGE_APP_CC) {
            // execution_cc.c:77: labels are vertex ids -- the caller's, or on a
            // symmetric graph the engine's, converted when the labels converge
            s.prop32[v] = g.sym ? (uint32_t)v : g.new2old[v];
            if (s.cc_best)
                s.cc_best[v] = NONE32;
        }
        else {
            s.prop64[v] = (g.weight_kind == WEDGE_WEIGHTS_F64) ? 0x7FF0000000000000ull : NONE64; /* execution_sssp.c:78 */
            if (s.dist32)
                s.dist32[v] = NONE32;
        }
    }
    const uint64_t nwords = (g.V + 31) / 32;
    for (uint64_t i = tid; i < nwords; i += stride) {
        s.front0[i] = 0u;
        if (s.front1)
            s.front1[i] = 0u;
    }
    const uint64_t cwords = ((uint64_t)g.T + 7) / 8;
    for (uint64_t i = tid; i < cwords; i += stride)
        s.chunk_bits[i] = 0u;
    const uint64_t swords = ((uint64_t)g.T / TILES_PER_REGION + 32) / 32;
    for (uint64_t i = tid; i < swords; i += stride)
        s.summary[i] = 0u;
    if (s.vis_c) {
        const uint64_t vwords = ((uint64_t)g.Vne + 31) / 32;
        for (uint64_t i = tid; i < vwords; i += stride)
            s.vis_c[i] = 0u;
    }
    if (s.tile_open) {
        const uint64_t owords = ((uint64_t)topen + 31) / 32;
        for (uint64_t i = tid; i < owords; i += stride) {
            const uint64_t left = (uint64_t)topen - i * 32;
            s.tile_open[i] = left >= 32 ? FULL : ((1u << left) - 1u);
        }
    }
    if (s.tile_need) {
        const uint64_t twords = (uint64_t)g.T / 32 + 2;
        for (uint64_t i = tid; i < twords; i += stride)
            s.tile_need[i] = 0u;
    }
    if (s.cand) {
        const uint64_t cwords = (uint64_t)g.Vne / 32 + 2;
        for (uint64_t i = tid; i < cwords; i += stride)
            s.cand[i] = 0u;
    }
}

// root activation (execution_bfs.c:110-117, execution_sssp.c:83-88) and the
// control block
__global__ void init_root_kernel(DevGraph g, DevState s, uint32_t app, uint64_t root_in, uint32_t sched,
                                 unsigned long long thr, uint32_t max_iter, uint32_t probe_iter, uint32_t probe_mode)
{
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t root = g.old2new[root_in]; /* the caller's id -> relabelled id */
    if (app == WEDGE_APP_BFS || app == WEDGE_APP_CC) {
        // BFS: the root is visited; CC: the vertex whose id is label 0 holds the least label already
        const uint32_t done = (app == WEDGE_APP_BFS) ? (uint32_t)root : g.sym ? 0u : g.old2new[0];
        if (tid == 0 && g.Vne) { /* its compressed index: dst_id ascends */
            uint32_t lo = 0, hi = g.Vne;
            while (lo < hi) {
                const uint32_t mid = lo + (hi - lo) / 2u;
                if (g.dst_id[mid] < done)
                    lo = mid + 1u;
                else
                    hi = mid;
            }
            if (lo < g.Vne && g.dst_id[lo] == done)
                atomicOr(&s.vis_c[lo >> 5], 1u << (lo & 31u));
        }
    }
    if (tid == 0) {
        Ctrl* c = s.ctrl;
        c->mass = 0;
        c->edges_scanned = 0;
        c->tiles_scanned = 0;
        c->dsts_scanned = 0;
        c->activated = 0;
        c->threshold = thr;
        c->items = 0;
        c->alist_n = 0;
        c->cand_n = 0;
        c->need_n = 0;
        c->tiles = 0;
        c->iter = 0;
        c->wedge_iters = 0;
        c->done = 0;
        c->not_converged = 0;
        c->max_iter = max_iter;
        c->sched = sched;
        c->parity = 0;
        c->loop = 1;
        c->error = 0;
        c->pull_launches = 0;
        c->probe_iter = probe_iter;
        c->probe_mode = probe_mode;
        c->learned_iters = 0;
        c->pr_total = 0.0;
        c->pr_sum = 0.0;
        c->probe_edges = s.probe_edges;
        c->narrow_ovf = 0;
        c->ovf_redo = 0;
        if (app == WEDGE_APP_CC) {
            c->last_mass = g.E;
            c->mode = MODE_DENSE; /* first CC pull is always dense, execution_cc.c:103 */
        } else {
            if (app == WEDGE_APP_SSSP) {
                s.prop64[root] = 0ull; /* 0.0 has the same bits */
                if (s.dist32)
                    s.dist32[root] = 0u;
            }
            s.front0[root >> 5] |= 1u << (root & 31u);
            c->last_mass = g.outdeg[root];
            c->mode = choose_mode(sched, g.outdeg[root], thr);
            if (sched == WEDGE_SCHED_PROBE && probe_iter == 0u)
                c->mode = probe_mode;
        }
        if (s.log) {
            for (int i = 0; i < 16; ++i)
                s.log[0].feat[i] = 0.0f; /* iteration 0 is chosen before any pull: no features */
            s.log[0].learned = 0u;
        }
        if (g.T == 0) {
            c->done = 1;
            c->loop = 0;
        }
    }
}

/* -------------------------------------------- CC label space (symmetric) */

// On a symmetric graph the labels converge to the least engine id of each
// component (its representative r); the reference's label is the least caller
// id of the component (execution_cc.c:77 and the min-pull of
// phase_edge_pull_cc.c).  best[r] = min over the component of new2old[v], with
// best preset to NONE32.  Label 0 (the component of engine vertex 0, the
// highest-degree vertex: the giant component) is reduced per block first;
// other components are small and take one global atomic per vertex.
__global__ void cc_best_kernel(DevGraph g, const uint32_t* label, uint32_t* best)
{
    __shared__ uint32_t best0;
    if (threadIdx.x == 0)
        best0 = NONE32;
    __syncthreads();
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    uint32_t m0 = NONE32;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < g.V; v += stride) {
        const uint32_t r = label[v], o = g.new2old[v];
        if (r == 0u)
            m0 = o < m0 ? o : m0;
        else
            atomicMin(&best[r], o);
    }
    m0 = __reduce_min_sync(FULL, m0);
    if ((threadIdx.x & 31) == 0 && m0 != NONE32)
        atomicMin(&best0, m0);
    __syncthreads();
    if (threadIdx.x == 0 && best0 != NONE32)
        atomicMin(&best[0], best0);
}

// label[v] = best[label[v]]: the caller-id labels
__global__ void cc_apply_kernel(DevGraph g, uint32_t* label, const uint32_t* best)
{
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < g.V; v += (uint64_t)gridDim.x * blockDim.x)
        label[v] = best[label[v]];
}

/* ------------------------------------------------------------- PageRank */

// 1 / outdegree' for every vertex (outdegree, or N for a dangling vertex;
// execution_pr.c:384-390), once per PageRank state: the vertex phase then
// multiplies where the reference divides (phase_vertex_pr.c:57-66), which this
// GPU's FP64 units make the phase's cost; the results differ by at most an ulp
// per step.
__global__ void pr_inv_outdeg_kernel(DevGraph g, double* inv_od)
{
    const double N = (double)g.V;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < g.V; v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t od = g.outdeg[v];
        inv_od[v] = __ddiv_rn(1.0, od ? (double)od : N);
    }
}

// execution_initialize_pr (execution_pr.c:380-392); max_iter bounds the
// captured iteration loop
__global__ void pr_init_kernel(DevGraph g, DevState s, uint32_t max_iter)
{
    const double invN = __ddiv_rn(1.0, (double)g.V);
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < g.V; v += (uint64_t)gridDim.x * blockDim.x) {
        s.acc[v] = 0.0;
        s.rank[v] = __dmul_rn(invN, s.inv_od[v]);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Ctrl* c = s.ctrl;
        c->iter = 0;
        c->wedge_iters = 0;
        c->edges_scanned = 0;
        c->tiles_scanned = 0;
        c->dsts_scanned = 0;
        c->activated = 0;
        c->pull_launches = 0;
        c->last_mass = 0;
        c->done = 0;
        c->mode = MODE_DENSE;
        c->parity = 0;
        c->need_n = 0;
        c->error = 0;
        c->pr_total = 0.0;
        c->pr_prev = 0.0;
        c->pr_sum = 0.0;
        c->max_iter = max_iter;
    }
}

// In-edge sums of the destinations whose in-edges span tiles: the partial sums
// of the tiles a destination continues through (tail(t), t0 <= t < t1), then the
// partial of the tile it ends in (head(t1)), in a fixed order (the GPU
// counterpart of the ordered merge of phases.c:71-114).  A thread sums each of
// the nshort splits at the front of the lists serially (most span one tile
// boundary); a warp sums each of the nwide at the back (hubs).
template <class Tail, class Head>
__device__ __forceinline__ void merge_splits(const DevGraph& g, double* acc, const uint32_t* split_k,
                                             const uint32_t* split_t0, const uint32_t* split_t1, uint32_t nshort,
                                             uint32_t nwide, uint32_t cap, Tail tail, Head head)
{
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthreads = gridDim.x * blockDim.x;
    for (uint32_t i = tid; i < nshort; i += nthreads) {
        const uint32_t t0 = split_t0[i], t1 = split_t1[i], k = split_k[i];
        double x = 0.0;
        for (uint32_t t = t0; t < t1; ++t)
            x = __dadd_rn(x, tail(t));
        acc[g.dst_ident ? k : g.dst_id[k]] = __dadd_rn(x, head(t1));
    }
    const int lane = threadIdx.x & 31;
    for (uint32_t j = tid >> 5; j < nwide; j += nthreads >> 5) {
        const uint32_t i = cap - 1u - j;
        const uint32_t a = split_t0[i], b = split_t1[i];
        // four independent sums per lane, combined in a fixed order
        double x0 = 0.0, x1 = 0.0, x2 = 0.0, x3 = 0.0;
        uint32_t t = a + lane;
        for (; t + 96u < b; t += 128u) {
            x0 = __dadd_rn(x0, tail(t));
            x1 = __dadd_rn(x1, tail(t + 32u));
            x2 = __dadd_rn(x2, tail(t + 64u));
            x3 = __dadd_rn(x3, tail(t + 96u));
        }
        for (; t < b; t += 32u)
            x0 = __dadd_rn(x0, tail(t));
        const double x = warp_sum_f64(__dadd_rn(__dadd_rn(x0, x1), __dadd_rn(x2, x3)));
        if (lane == 0) {
            const uint32_t k = split_k[i];
            acc[g.dst_ident ? k : g.dst_id[k]] = __dadd_rn(x, head(b));
        }
    }
}

// The iteration's counters and log record, and the in-edge sums of the
// destinations that span tiles (fixed tile order; the GPU counterpart of the
// ordered merge of phases.c:71-114).
__global__ void pr_finish_kernel(DevGraph g, DevState s, uint32_t nblocks, const unsigned long long* block_cnt)
{
    Ctrl* c = s.ctrl;
    if (blockIdx.x == 0) {
        unsigned long long cnt[NCNT];
        reduce_counters(block_cnt, nblocks, cnt); /* contains __syncthreads */
        if (threadIdx.x == 0) {
            c->last_mass = 0;
            log_iteration(s, c, cnt);
        }
    }
    merge_splits(g, s.acc, g.split_k, g.split_t0, g.split_t1, g.nsplit, g.nwide, g.T, [&](uint32_t t) { return s.tail_part[t]; },
                 [&](uint32_t t) { return s.head_part[t]; });
}

// perform_vertex_phase_pr (phase_vertex_pr.c:26-77):
// rank' = ((acc + (1 - total)/N) * d + (1 - d)/N) / outdegree'
// (a multiply by s.inv_od where the state holds it; the no-alloc entry point,
// which has no state, divides)
__global__ void pr_vertex_kernel(DevGraph g, DevState s)
{
    const double N = (double)g.V;
    const double d = s.damping;
    const double omd = __ddiv_rn(__dsub_rn(1.0, d), N);
    const double corr = __ddiv_rn(__dsub_rn(1.0, s.ctrl->pr_total), N);
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < g.V; v += (uint64_t)gridDim.x * blockDim.x) {
        const double x = __dadd_rn(__dmul_rn(__dadd_rn(s.acc[v], corr), d), omd);
        if (s.inv_od) {
            s.rank[v] = __dmul_rn(x, s.inv_od[v]);
        } else {
            const uint32_t od = g.outdeg[v];
            s.rank[v] = __ddiv_rn(x, od ? (double)od : N);
        }
    }
}

// Total rank: the sum of all accumulators after the merge.  The reference
// sums the gathered values per thread during the edge phase and combines the
// per-thread sums (phases.c:37-46, phase_vertex_pr.c:43-46); this is the same
// quantity summed in another fixed order, once per vertex instead of once per
// edge (FP64 additions are scarce on this GPU).  Each block writes its sum to
// part[]; the last block to finish combines them in block order.  grid <=
// the length of part[].
__global__ void pr_total_kernel(const double* acc, uint64_t V, double* part, Ctrl* c)
{
    __shared__ double sh[AUX_THREADS / 32];
    __shared__ unsigned int ticket;
    const int lane = threadIdx.x & 31;
    const uint64_t n = (uint64_t)gridDim.x * blockDim.x;
    uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    double x0 = 0.0, x1 = 0.0, x2 = 0.0, x3 = 0.0;
    for (; v + 3u * n < V; v += 4u * n) {
        x0 = __dadd_rn(x0, acc[v]);
        x1 = __dadd_rn(x1, acc[v + n]);
        x2 = __dadd_rn(x2, acc[v + 2u * n]);
        x3 = __dadd_rn(x3, acc[v + 3u * n]);
    }
    for (; v < V; v += n)
        x0 = __dadd_rn(x0, acc[v]);
    double x = warp_sum_f64(__dadd_rn(__dadd_rn(x0, x1), __dadd_rn(x2, x3)));
    if (lane == 0)
        sh[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < AUX_THREADS / 32; ++w)
            t = __dadd_rn(t, sh[w]);
        part[blockIdx.x] = t;
        __threadfence();
        ticket = atomicAdd(&c->pr_ticket, 1u);
    }
    __syncthreads();
    if (ticket == gridDim.x - 1u && threadIdx.x < 32) { /* the last block: every part[] is visible */
        __threadfence();
        double y = 0.0;
        for (uint32_t i = lane; i < gridDim.x; i += 32u)
            y = __dadd_rn(y, __ldcg(part + i));
        y = warp_sum_f64(y);
        if (lane == 0) {
            c->pr_total = y;
            c->pr_ticket = 0u;
        }
    }
}

/* -------------------------------------------- compensated-FP32 PageRank */
//
// WEDGE_PREC_FP32C: ranks, gathers, per-destination sums and the vertex phase
// in FP32; FP64 only for the total rank S, whose (1 - S)/N term renormalises
// the dangling mass (phase_vertex_pr.c:57-72).  The reference computes S as
// the sum of all accumulators after the edge phase (phases.c:37-46).  Since
//     S(i) = sum_v acc_v(i) = sum_{s : outdeg_s > 0} rank_s(i-1),
// the total an iteration needs is known when its pull starts: the previous
// iteration sums its new non-dangling ranks.  So the vertex phase runs inside
// the pull, once per destination, as soon as the destination's sum is
// complete, and nothing per vertex is written twice:
//   pr32_pull_kernel    tiles of PR32_TILE in-edges; a destination inside one
//                       tile gets its new rank there (staged per warp in shared
//                       memory, then written by the warp's lanes together)
//   pr32_finish_kernel  destinations spanning tiles (two-sum of the per-tile
//                       partials in tile order) and vertices with out-edges but
//                       no in-edges (all take the same rank)
//   pr32_total_kernel   S of the next iteration from the per-block FP64 sums
// Ranks are double-buffered by iteration parity; vertices with neither in- nor
// out-edges are written once, after the last iteration (pr32_iso_kernel).
constexpr int PR32_EPL = 16;
constexpr uint32_t PR32_TILE = 32u * PR32_EPL;
// staged destination sums per warp: 128 cover every destination of 97% of the
// 512-edge tiles of an R-MAT graph; the shared memory they take comes out of
// the L1 the gathers depend on (a stage of a whole tile's 512 ran 0.5 ms per
// iteration slower at R-MAT scale 26)
constexpr uint32_t PR32_SLOTS = 128;

__device__ __forceinline__ const float* pr32_cur(const DevState& s)
{
    return s.rank32 + ((s.ctrl->iter & 1u) ? s.rstride : 0ull);
}

// FP32 constants of one iteration's vertex phase: rank' = (acc + corr)*d + omd
struct Pr32K {
    float corr, d, omd;
};

__device__ __forceinline__ Pr32K pr32_constants(const DevGraph& g, const DevState& s, double total)
{
    const double N = (double)g.V;
    Pr32K k;
    k.corr = __double2float_rn(__ddiv_rn(__dsub_rn(1.0, total), N));
    k.d = __double2float_rn(s.damping);
    k.omd = __double2float_rn(__ddiv_rn(__dsub_rn(1.0, s.damping), N));
    return k;
}

// the vertex phase of one vertex (phase_vertex_pr.c:72) in FP32: its rank
// (before the division by outdegree') from its in-edge sum
__device__ __forceinline__ float pr32_rank(const Pr32K& k, float sum)
{
    return __fmaf_rn(__fadd_rn(sum, k.corr), k.d, k.omd);
}

__device__ __forceinline__ F2 f2_add(F2 a, float x) { return AddF2()(a, F2{x, 0.0f}); }

// FP64 sum of a block's per-thread (sum, compensation) pairs, in a fixed
// order; returned on thread 0.  blockDim.x is a multiple of 32, at most 1024.
__device__ __forceinline__ double block_sum_f2(F2 x)
{
    __shared__ double sh[32];
    double v = warp_sum_f64(__dadd_rn((double)x.s, (double)x.c));
    if ((threadIdx.x & 31) == 0)
        sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x == 0)
        for (uint32_t w = 0; w < blockDim.x / 32u; ++w)
            t = __dadd_rn(t, sh[w]);
    return t;
}

// 1/outdegree' in FP32 (the reference divides by outdegree, or by N for a
// dangling vertex: execution_pr.c:384-390); negative marks a dangling vertex
__global__ void pr32_inv_kernel(DevGraph g, float* inv32)
{
    const double N = (double)g.V;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < g.V; v += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t od = g.outdeg[v];
        inv32[v] = od ? __double2float_rn(__ddiv_rn(1.0, (double)od)) : -__double2float_rn(__ddiv_rn(1.0, N));
    }
}

// flags of the vertices without in-edges: 1 with out-edges (zlist), 2 without (ilist)
__global__ void pr32_noin_flags_kernel(DevGraph g, const uint32_t* has_in, uint32_t* fz, uint32_t* fi)
{
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < g.V; v += (uint64_t)gridDim.x * blockDim.x) {
        const bool noin = !((has_in[v >> 5] >> (v & 31u)) & 1u);
        fz[v] = (noin && g.outdeg[v] != 0u) ? 1u : 0u;
        fi[v] = (noin && g.outdeg[v] == 0u) ? 1u : 0u;
    }
}

__global__ void mark_has_in_kernel(DevGraph g, uint32_t* has_in)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < g.Vne; k += gridDim.x * blockDim.x) {
        const uint32_t v = g.dst_ident ? k : g.dst_id[k];
        atomicOr(&has_in[v >> 5], 1u << (v & 31u));
    }
}

// complete destinations past the first PR32_SLOTS of their PR32_TILE-edge
// tile (they are finished from ovf_sum): their count per tile (fill == null)
// or, at the tile's offset from a scan of the counts, the list itself in tile
// order.  The tile geometry is the pull's (the destination-start bitmap).
__global__ void pr32_overflow_kernel(DevGraph g, uint32_t T, uint32_t* count, const uint32_t* off, uint32_t* fill)
{
    constexpr uint32_t W = PR32_TILE / 32, Q = PR32_TILE / TILE;
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < T; t += gridDim.x * blockDim.x) {
        const uint64_t w0 = (uint64_t)t * W;
        uint32_t starts = 0;
        for (uint32_t i = 0; i < W; ++i)
            starts += __popc(g.dst_start[w0 + i]);
        const bool fresh = g.dst_start[w0] & 1u;
        const uint32_t nd = starts - (fresh ? 1u : 0u) + 1u;
        const uint32_t k0 = g.tile_dst0[(uint64_t)t * Q], kend = g.tile_dst0[((uint64_t)t + 1u) * Q];
        const bool tail_cont = t + 1u < T && kend == k0 + nd - 1u;
        const uint32_t jlo = max(fresh ? 0u : 1u, PR32_SLOTS);
        const uint32_t jhi = tail_cont ? nd - 1u : nd;
        const uint32_t n = jhi > jlo ? jhi - jlo : 0u;
        if (!fill) {
            count[t] = n;
        } else {
            for (uint32_t j = 0; j < n; ++j)
                fill[off[t] + j] = k0 + jlo + j;
        }
    }
}

// stream compaction by an exclusive scan of 0/1 flags: list in ascending id order
__global__ void compact_flags_kernel(const uint32_t* flag, const uint32_t* pos, uint64_t n, uint32_t* list)
{
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < n; v += (uint64_t)gridDim.x * blockDim.x)
        if (flag[v])
            list[pos[v]] = (uint32_t)v;
}

// execution_initialize_pr (execution_pr.c:380-392) in FP32: rank = 1/N, stored
// divided by outdegree'; the per-block sums of the non-dangling ranks give the
// total of iteration 0 (pr32_total_kernel)
__global__ void pr32_init_kernel(DevGraph g, DevState s, uint32_t max_iter)
{
    const float r = __double2float_rn(__ddiv_rn(1.0, (double)g.V));
    F2 m{0.0f, 0.0f};
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < g.V; v += (uint64_t)gridDim.x * blockDim.x) {
        const float inv = s.inv32[v];
        s.rank32[v] = __fmul_rn(r, fabsf(inv));
        if (inv > 0.0f)
            m = f2_add(m, r);
    }
    const double t = block_sum_f2(m);
    if (threadIdx.x == 0)
        s.pmass[blockIdx.x] = t;
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        Ctrl* c = s.ctrl;
        c->iter = 0;
        c->wedge_iters = 0;
        c->edges_scanned = 0;
        c->tiles_scanned = 0;
        c->dsts_scanned = 0;
        c->activated = 0;
        c->pull_launches = 0;
        c->last_mass = 0;
        c->done = 0;
        c->mode = MODE_DENSE;
        c->parity = 0;
        c->need_n = 0;
        c->error = 0;
        c->pr_total = 0.0;
        c->pr_prev = 0.0;
        c->pr_sum = 0.0;
        c->max_iter = max_iter;
    }
}

// The edge pull and, for every destination whose in-edges lie in one tile, the
// vertex phase (perform_edge_pull_phase_pr, phase_edge_pull_pr.c:28-116, and
// perform_vertex_phase_pr, phase_vertex_pr.c:26-77).  One 1024-thread block per
// SM; a warp takes tiles of PR32_TILE in-edges in a static stride: 16 sources
// per lane in two 256-bit loads, their ranks gathered from the hub cache (the
// low-id end of the rank array, bulk-copied into shared memory at launch) or
// global memory, folded per destination by the segmented two-sum reduction.
// The sums of the tile's complete destinations are staged in the warp's slice
// of shared memory and finished by the warp's lanes together: consecutive
// destinations, so their outdegree' and rank writes coalesce.  Destinations
// spanning tiles leave (sum, compensation) partials for pr32_finish_kernel.
// Dynamic shared memory: hub cache (hub_bytes) | staged sums [32 warps][PR32_SLOTS].
// block_cnt[NCNT*b + CNT_*] as pull_kernel's; s.pmass[b] = the block's sum of
// the new non-dangling ranks.
__global__ void __launch_bounds__(PULL_THREADS, 1) pr32_pull_kernel(DevGraph g, DevState s, unsigned long long* block_cnt)
{
    constexpr int EPL = PR32_EPL;
    constexpr int WARPS = PULL_THREADS / 32;
    constexpr uint32_t Q = PR32_TILE / TILE; /* 128-edge index entries per tile */
    __shared__ unsigned long long sh_cnt[WARPS][3];
    __shared__ unsigned long long hub_bar;
    extern __shared__ __align__(16) unsigned char pr32_smem[];
    const Ctrl* c = s.ctrl;
    const uint32_t par = c->iter & 1u;
    const float* cur = s.rank32 + (par ? s.rstride : 0ull);
    float* nxt = s.rank32 + (par ? 0ull : s.rstride);
    const Pr32K K = pr32_constants(g, s, c->pr_total);
    const int lane = threadIdx.x & 31;
    const int wib = threadIdx.x >> 5;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nw = (gridDim.x * blockDim.x) >> 5;
    const uint32_t T = (uint32_t)((g.E + PR32_TILE - 1) / PR32_TILE); /* tiles holding real in-edges */
    const uint32_t hub_bytes = s.hub_bytes;
    const float* hub = reinterpret_cast<const float*>(pr32_smem);
    float* my_sum = reinterpret_cast<float*>(pr32_smem + hub_bytes) + (uint32_t)wib * PR32_SLOTS;

    // ---- hub cache: ranks [0, hub_n) of the current buffer
    const bool use_hub = hub_bytes != 0u && (s.rstride & 3ull) == 0ull;
    if (use_hub) {
        if (threadIdx.x == 0) {
            mbar_init(&hub_bar, 1u);
            mbar_arrive_expect_tx(&hub_bar, hub_bytes);
            for (uint32_t off = 0; off < hub_bytes; off += 32768u)
                bulk_g2s(pr32_smem + off, reinterpret_cast<const unsigned char*>(cur) + off, min(32768u, hub_bytes - off),
                         &hub_bar);
        }
        __syncthreads();
    }
    uint32_t hub_lim = 0; /* cache entries this warp reads: 0 until the copy completed */

    unsigned long long edges = 0, tiles = 0, dsts = 0;
    F2 mass{0.0f, 0.0f};
    const unsigned long long pol = l2_evict_first_policy();
    uint32_t t = gw;
    uint32_t k0n = 0, kendn = 0;
    if (t < T) {
        k0n = g.tile_dst0[(uint64_t)t * Q];
        kendn = g.tile_dst0[((uint64_t)t + 1u) * Q];
    }
    for (; t < T; t += nw) {
        const uint32_t k0 = k0n, kend = kendn;
        if (t + nw < T) { /* the next tile's bounds, one tile ahead */
            k0n = g.tile_dst0[(uint64_t)(t + nw) * Q];
            kendn = g.tile_dst0[((uint64_t)(t + nw) + 1u) * Q];
        }
        if (use_hub && hub_lim == 0u) {
            uint32_t ready = 0u;
            if (lane == 0)
                ready = mbar_test_wait(&hub_bar, 0u) ? 1u : 0u;
            if (__shfl_sync(FULL, ready, 0))
                hub_lim = hub_bytes / 4u;
        }
        ++tiles;
        const uint64_t base = (uint64_t)t * PR32_TILE;
        uint32_t sa[EPL];
        {
            const uint32_t* p = g.src + base + (uint64_t)lane * EPL;
            uint32_t x[8];
            ld_stream_v8_ef(p, x, pol); /* read once: evict first, the ranks stay in L2 */
#pragma unroll
            for (int j = 0; j < 8; ++j)
                sa[j] = x[j];
            ld_stream_v8_ef(p + 8, x, pol);
#pragma unroll
            for (int j = 0; j < 8; ++j)
                sa[8 + j] = x[j];
        }
        F2 v[EPL];
#pragma unroll
        for (int q = 0; q < EPL; ++q) {
            const uint32_t x = sa[q];
            v[q] = F2{(x < hub_lim) ? hub[x] : (x != NONE32) ? ld_ro_f32(cur + x) : 0.0f, 0.0f};
        }
        if (lane == 0) /* in-edges of the tile: all but the padding after the last one */
            edges += (g.E - base < PR32_TILE) ? g.E - base : PR32_TILE;
        TileGeo<EPL> tg;
        tile_geometry_bits<EPL>(g, base, t + 1u >= T, k0, kend, lane, tg);
        dsts += tg.ndst;
        // The reduction stages the sums of the tile's first PR32_SLOTS complete
        // destinations; the vertex phase then runs for them with the lanes over
        // consecutive destinations.  A tile of more destinations (many low
        // in-degree ones) leaves the others' sums in ovf_sum, finished by
        // pr32_finish_kernel from the graph's fixed list of such destinations.
        seg_reduce<EPL>(v, tg, lane, AddF2(), [&](uint32_t k, F2 val, int kind) {
            if (kind == EMIT_COMPLETE) {
                const uint32_t slot = k - tg.k0;
                if (slot < PR32_SLOTS)
                    my_sum[slot] = __fadd_rn(val.s, val.c);
                else
                    s.ovf_sum[k] = __fadd_rn(val.s, val.c);
            } else {
                (kind == EMIT_HEAD ? s.phead : s.ptail)[t] = make_float2(val.s, val.c);
            }
        });
        __syncwarp();
        const uint32_t nd = tg.ndst;
        const uint32_t jlo = tg.k0_fresh ? 0u : 1u;                        /* slot 0 began in an earlier tile */
        const uint32_t jhi = min(tg.tail_cont ? nd - 1u : nd, PR32_SLOTS); /* the last slot may continue */
        for (uint32_t j = jlo + (uint32_t)lane; j < jhi; j += 32u) {
            const uint32_t k = tg.k0 + j;
            const uint32_t vtx = g.dst_ident ? k : g.dst_id[k];
            const float inv = s.inv32[vtx];
            const float r = pr32_rank(K, my_sum[j]);
            nxt[vtx] = __fmul_rn(r, fabsf(inv));
            if (inv > 0.0f)
                mass = f2_add(mass, r);
        }
        __syncwarp(); /* my_sum is rewritten by the next tile */
    }
    // the block may not retire with its bulk copy in flight
    if (use_hub && threadIdx.x == 0 && !mbar_wait_bounded(&hub_bar, 0u, HUB_WAIT_TRIES)) {
        atomicOr(&s.ctrl->error, ERR_HUB_TIMEOUT);
        mbar_wait_bounded(&hub_bar, 0u, HUB_WAIT_TRIES);
    }
    edges = warp_sum_u64(edges);
    if (lane == 0) {
        sh_cnt[wib][0] = edges;
        sh_cnt[wib][1] = tiles; /* warp-uniform */
        sh_cnt[wib][2] = dsts;  /* warp-uniform */
    }
    const double bm = block_sum_f2(mass); /* contains __syncthreads */
    if (threadIdx.x == 0)
        s.pmass[blockIdx.x] = bm;
    if (threadIdx.x < NCNT) {
        unsigned long long a = 0;
        if (threadIdx.x == CNT_EDGES || threadIdx.x == CNT_TILES || threadIdx.x == CNT_DSTS) {
            const int col = threadIdx.x == CNT_EDGES ? 0 : threadIdx.x == CNT_TILES ? 1 : 2;
            for (int w = 0; w < WARPS; ++w)
                a += sh_cnt[w][col];
        }
        block_cnt[NCNT * blockIdx.x + threadIdx.x] = a;
    }
}

// Destinations whose in-edges span tiles: the (sum, compensation) partials of
// the tiles they continue through, then of the tile they end in, combined by
// two-sum in tile order (the counterpart of the ordered merge of
// phases.c:71-114), then their vertex phase; and the vertices with out-edges
// but no in-edges, whose sum is 0.  Short splits take a thread each, long ones
// (hubs) a warp each.  s.pmass[part0 + b] = the block's sum of new non-dangling ranks.
__global__ void pr32_finish_kernel(DevGraph g, DevState s, uint32_t part0)
{
    const Ctrl* c = s.ctrl;
    float* nxt = s.rank32 + ((c->iter & 1u) ? 0ull : s.rstride);
    const Pr32K K = pr32_constants(g, s, c->pr_total);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t nthr = gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    F2 mass{0.0f, 0.0f};
    auto finish = [&](uint32_t k, F2 sum) {
        const uint32_t vtx = g.dst_ident ? k : g.dst_id[k];
        const float inv = s.inv32[vtx];
        const float r = pr32_rank(K, __fadd_rn(sum.s, sum.c));
        nxt[vtx] = __fmul_rn(r, fabsf(inv));
        if (inv > 0.0f)
            mass = f2_add(mass, r);
    };
    const AddF2 add;
    for (uint32_t i = tid; i < s.pnsplit; i += nthr) {
        const uint32_t t0 = s.psplit_t0[i], t1 = s.psplit_t1[i];
        F2 x{0.0f, 0.0f};
        for (uint32_t tt = t0; tt < t1; ++tt) {
            const float2 p = s.ptail[tt];
            x = add(x, F2{p.x, p.y});
        }
        const float2 h = s.phead[t1];
        finish(s.psplit_k[i], add(x, F2{h.x, h.y}));
    }
    for (uint32_t j = tid >> 5; j < s.pnwide; j += nthr >> 5) {
        const uint32_t i = s.pT - 1u - j;
        const uint32_t a = s.psplit_t0[i], b = s.psplit_t1[i];
        F2 x{0.0f, 0.0f};
        for (uint32_t tt = a + (uint32_t)lane; tt < b; tt += 32u) {
            const float2 p = s.ptail[tt];
            x = add(x, F2{p.x, p.y});
        }
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) /* butterfly: the same fixed order on every run */
            x = add(x, F2{__shfl_xor_sync(FULL, x.s, d), __shfl_xor_sync(FULL, x.c, d)});
        if (lane == 0) {
            const float2 h = s.phead[b];
            finish(s.psplit_k[i], add(x, F2{h.x, h.y}));
        }
    }
    for (uint32_t i = tid; i < s.novf; i += nthr) { /* complete destinations past a tile's staged slots */
        const uint32_t k = s.ovf_list[i];
        finish(k, F2{s.ovf_sum[k], 0.0f});
    }
    const float r0 = pr32_rank(K, 0.0f);
    for (uint32_t i = tid; i < s.nz; i += nthr) {
        const uint32_t v = s.zlist[i];
        nxt[v] = __fmul_rn(r0, s.inv32[v]); /* out-edges: inv32 > 0 */
        mass = f2_add(mass, r0);
    }
    const double bm = block_sum_f2(mass);
    if (threadIdx.x == 0)
        s.pmass[part0 + blockIdx.x] = bm;
}

// The total rank the next iteration uses: the per-block FP64 sums in block
// order (one block of AUX_THREADS).  With nblocks > 0 the iteration is also
// counted and logged from the pull's block counters.
__global__ void pr32_total_kernel(DevState s, uint32_t nparts, const unsigned long long* block_cnt, uint32_t nblocks)
{
    __shared__ double sh[AUX_THREADS / 32];
    Ctrl* c = s.ctrl;
    double x = 0.0;
    for (uint32_t i = threadIdx.x; i < nparts; i += blockDim.x)
        x = __dadd_rn(x, s.pmass[i]);
    x = warp_sum_f64(x);
    if ((threadIdx.x & 31) == 0)
        sh[threadIdx.x >> 5] = x;
    __syncthreads();
    unsigned long long cnt[NCNT];
    if (nblocks)
        reduce_counters(block_cnt, nblocks, cnt); /* uniform branch; contains __syncthreads */
    if (threadIdx.x == 0) {
        double S = 0.0;
        for (int w = 0; w < AUX_THREADS / 32; ++w)
            S = __dadd_rn(S, sh[w]);
        c->pr_prev = c->pr_total;
        c->pr_total = S;
        if (nblocks) {
            c->last_mass = 0;
            log_iteration(s, c, cnt);
        }
    }
}

// After the last iteration: the vertices with neither in- nor out-edges, whose
// rank is the same constant and which no pull gathers, in the last buffer
// written (nothing before the first iteration: the initial ranks stand)
__global__ void pr32_iso_kernel(DevGraph g, DevState s)
{
    const Ctrl* c = s.ctrl;
    if (c->iter == 0u)
        return;
    float* last = s.rank32 + ((c->iter & 1u) ? s.rstride : 0ull);
    const float r0 = pr32_rank(pr32_constants(g, s, c->pr_prev), 0.0f);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < s.ni; i += gridDim.x * blockDim.x) {
        const uint32_t v = s.ilist[i];
        last[v] = __fmul_rn(r0, fabsf(s.inv32[v]));
    }
}

// condition of the captured PageRank iteration loop
__global__ void pr_loop_cond_kernel(DevState s, cudaGraphConditionalHandle handle)
{
    cudaGraphSetConditional(handle, s.ctrl->iter < s.ctrl->max_iter ? 1u : 0u);
}

// PageRank Sum (execution_pr.c:63-71): sum of rank' * outdegree' over all vertices
__global__ void pr_sum_kernel(DevGraph g, DevState s, double* block_out)
{
    __shared__ double sh[AUX_THREADS / 32];
    const double N = (double)g.V;
    const bool c32 = s.precision == WEDGE_PREC_FP32C;
    const float* r32 = c32 ? pr32_cur(s) : nullptr;
    double x = 0.0;
    if (c32) {
        // compensated FP32 per thread (this GPU's FP64 units are slow), FP64 across threads
        const float Nf = (float)g.V;
        F2 a{0.0f, 0.0f};
        for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < g.V; v += (uint64_t)gridDim.x * blockDim.x) {
            const uint32_t od = g.outdeg[v];
            a = f2_add(a, __fmul_rn(r32[v], od ? (float)od : Nf));
        }
        x = __dadd_rn((double)a.s, (double)a.c);
    } else {
        for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < g.V; v += (uint64_t)gridDim.x * blockDim.x) {
            const uint32_t od = g.outdeg[v];
            x = __dadd_rn(x, __dmul_rn(s.rank[v], od ? (double)od : N));
        }
    }
    x = warp_sum_f64(x);
    if ((threadIdx.x & 31) == 0)
        sh[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < AUX_THREADS / 32; ++w)
            t = __dadd_rn(t, sh[w]);
        block_out[blockIdx.x] = t;
    }
}

__global__ void pr_sum_final_kernel(DevState s, const double* block_out, uint32_t n)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double t = 0.0;
        for (uint32_t i = 0; i < n; ++i)
            t = __dadd_rn(t, block_out[i]);
        s.ctrl->pr_sum = t;
    }
}

/* --------------------------------------------------------------- results */

// graph_vertex_props in the reference's representation (one 64-bit word per vertex)
__global__ void export_kernel(DevGraph g, DevState s, uint32_t app, unsigned long long* out)
{
    for (uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; o < g.V; o += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = g.old2new[o]; /* results come back in the caller's numbering */
        unsigned long long x;
        if (app == WEDGE_APP_BFS) {
            const uint32_t p = s.prop32[v];
            x = (p == NONE32) ? NONE64 : (unsigned long long)g.new2old[p];
        } else if (app == WEDGE_APP_CC) {
            const uint32_t l = s.prop32[v];
            x = (unsigned long long)__double_as_longlong((double)(s.cc_map ? s.cc_map[l] : l));
        } else if (app == WEDGE_APP_SSSP) {
            x = s.prop64[v];
        } else {
            x = (unsigned long long)__double_as_longlong(s.precision == WEDGE_PREC_FP32C ? (double)pr32_cur(s)[v] : s.rank[v]);
        }
        out[o] = x;
    }
}

// -o output on the device (source/main.c:112-150): "%llu %s\n" per vertex, with
// the value as execution_get_vertex_prop_string_{bfs,cc,sssp} print it:
// BFS and SSSP "%lld" of the 64-bit word (UINT64_MAX prints -1), CC "%.0lf" of
// an integer label (exact).  A length pass, an exclusive scan, a write pass.
__device__ __forceinline__ void out_value(const DevGraph& g, const DevState& s, uint32_t app, uint64_t o, bool& neg,
                                          unsigned long long& x)
{
    const uint32_t v = g.old2new[o];
    neg = false;
    if (app == WEDGE_APP_BFS) {
        const uint32_t p = s.prop32[v];
        neg = p == NONE32;
        x = neg ? 1ull : (unsigned long long)g.new2old[p];
    } else if (app == WEDGE_APP_CC) {
        const uint32_t l = s.prop32[v];
        x = s.cc_map ? s.cc_map[l] : l;
    } else {
        const unsigned long long d = s.prop64[v];
        neg = (long long)d < 0;
        x = neg ? (unsigned long long)(-(long long)d) : d;
    }
}

__device__ __forceinline__ uint32_t dec_len(unsigned long long x)
{
    uint32_t n = 1;
    while (x >= 10ull) {
        x /= 10ull;
        ++n;
    }
    return n;
}

__device__ __forceinline__ void dec_put(char* p, unsigned long long x, uint32_t n)
{
    for (uint32_t i = n; i-- > 0;) {
        p[i] = (char)('0' + (int)(x % 10ull));
        x /= 10ull;
    }
}

__global__ void out_len_kernel(DevGraph g, DevState s, uint32_t app, unsigned long long* len)
{
    for (uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; o < g.V; o += (uint64_t)gridDim.x * blockDim.x) {
        bool neg;
        unsigned long long x;
        out_value(g, s, app, o, neg, x);
        len[o] = dec_len(o) + 1u + (neg ? 1u : 0u) + dec_len(x) + 1u;
    }
}

__global__ void out_write_kernel(DevGraph g, DevState s, uint32_t app, const unsigned long long* off, char* buf)
{
    for (uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; o < g.V; o += (uint64_t)gridDim.x * blockDim.x) {
        bool neg;
        unsigned long long x;
        out_value(g, s, app, o, neg, x);
        char* p = buf + off[o];
        const uint32_t n0 = dec_len(o);
        dec_put(p, o, n0);
        p += n0;
        *p++ = ' ';
        if (neg)
            *p++ = '-';
        const uint32_t n1 = dec_len(x);
        dec_put(p, x, n1);
        p[n1] = '\n';
    }
}

__global__ void export_outdeg_kernel(DevGraph g, unsigned long long* out)
{
    for (uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; o < g.V; o += (uint64_t)gridDim.x * blockDim.x)
        out[o] = g.outdeg[g.old2new[o]];
}

// first tile of the second dense-pull launch: the tile holding the first
// in-edge of the first destination with id >= hub_n, rounded up, so no tile of
// that launch writes a cached value (dst_id is ascending)
__global__ void hub_split_kernel(DevGraph g, uint32_t hub_n, uint32_t tile_e, uint32_t* out)
{
    uint32_t lo = 0, hi = g.Vne;
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2u;
        if (g.dst_id[mid] < hub_n)
            lo = mid + 1u;
        else
            hi = mid;
    }
    const unsigned long long pos = g.dst_off[lo]; /* dst_off[Vne] = E */
    out[0] = (uint32_t)((pos + tile_e - 1u) / tile_e);
    out[1] = lo; /* compressed destinations with ids < hub_n */
}

/* ================================================================ host */

int compute_grids(wedge_graph* h)
{
    int blocks = 0;
    WEDGE_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, pull_kernel<WEDGE_APP_CC, PullEpl<WEDGE_APP_CC>::value>, PULL_THREADS, 0));
    if (blocks < 1)
        return WEDGE_ERR_CUDA;
    h->pull_grid = (uint32_t)h->num_sms; /* one block per SM: the hub cache takes the SM's shared memory */
    h->build_grid = (uint32_t)h->num_sms * 8u;
    int dblocks = 0;
    WEDGE_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&dblocks, dst_kernel<WEDGE_APP_CC, PullEpl<WEDGE_APP_CC>::value>,
                                                              PULL_THREADS, 0));
    h->dst_grid = (uint32_t)h->num_sms * (uint32_t)(dblocks < 1 ? 1 : dblocks > 2 ? 2 : dblocks);
    return WEDGE_OK;
}

// block-counter slots: the launches of the largest pull (CC: two dst_kernel
// launches + two tile launches)
static uint64_t counter_slots(const wedge_graph* h) { return 2ull * h->dst_grid + 2ull * h->pull_grid; }

// Launch knobs: the value set on the handle, else its environment variable,
// else the default.  Values outside a knob's range read as unset.
static bool knob_ok(int k, uint64_t v)
{
    switch (k) {
    case WEDGE_KNOB_HUB_BYTES:
        return v <= 196608u && v % 16u == 0u;
    case WEDGE_KNOB_PROBE_EDGES:
        return v >= 1u && v <= 4096u;
    case WEDGE_KNOB_SSSP_TILE:
        return v == 256u || v == 512u;
    case WEDGE_KNOB_SSSP_NARROW:
        return v <= 0xFFFFFFFEull;
    default:
        return false;
    }
}

constexpr uint64_t HUB_BYTES_DEFAULT = 65536;

static uint64_t knob_value(const wedge_graph* h, int k)
{
    static const uint64_t defaults[WEDGE_KNOBS] = {HUB_BYTES_DEFAULT, PROBE_EDGES, 512u, 1u};
    if (h->knob[k] != WEDGE_KNOB_DEFAULT)
        return h->knob[k];
    const char* e = nullptr;
    uint64_t v = 0;
    switch (k) {
    case WEDGE_KNOB_HUB_BYTES:
        e = getenv("WEDGE_HUB_BYTES");
        break;
    case WEDGE_KNOB_PROBE_EDGES:
        e = getenv("WEDGE_PROBE_EDGES");
        break;
    case WEDGE_KNOB_SSSP_TILE: {
        // default: 512-edge tiles from 2^23 in-edges; below, the extra launches of
        // the 512-edge pull (two instantiations and a finish per launch) cost more
        // than its faster tiles save (batched workload, scales 12-20: 181 against
        // 156 ms one query at a time)
        const char* t = getenv("WEDGE_SSSP_TILES512");
        return (t && t[0] == '0') ? 256u : (t && t[0] == '1') ? 512u : h->g.E >= (1ull << 23) ? 512u : 256u;
    }
    case WEDGE_KNOB_SSSP_NARROW:
        e = getenv("WEDGE_SSSP_NARROW");
        break;
    default:
        return 0;
    }
    if (!e || !*e)
        return defaults[k];
    char* end = nullptr;
    v = strtoull(e, &end, 10);
    return (end && *end == '\0' && knob_ok(k, v)) ? v : defaults[k];
}

// SSSP runs sssp_pull_kernel (512-edge tiles) where the knob asks for it and
// the graph has byte-wide weights and in-edge positions, else pull_kernel
// (256-edge tiles; 20.6 against 23.2 ms per SSSP at R-MAT scale 26 with
// 64-bit distance gathers)
static bool sssp_tiles512(const wedge_graph* h)
{
    return h->s.push && h->g.w8 && knob_value(h, WEDGE_KNOB_SSSP_TILE) == 512u;
}
static uint32_t sssp_split_grid(wedge_graph* h);

static const void* pull_fn(const wedge_graph* h, int app)
{
    if (app == WEDGE_APP_SSSP && sssp_tiles512(h))
        return (const void*)sssp_pull_kernel<false>;
    switch (app) {
    case WEDGE_APP_BFS:
        return (const void*)pull_kernel<WEDGE_APP_BFS, PullEpl<WEDGE_APP_BFS>::value>;
    case WEDGE_APP_CC:
        return (const void*)pull_kernel<WEDGE_APP_CC, PullEpl<WEDGE_APP_CC>::value>;
    case WEDGE_APP_SSSP:
        return (const void*)pull_kernel<WEDGE_APP_SSSP, PullEpl<WEDGE_APP_SSSP>::value>;
    default:
        return (const void*)pull_kernel<WEDGE_APP_PR, PullEpl<WEDGE_APP_PR>::value>;
    }
}

static uint32_t pull_tile_e(const wedge_graph* h, int app)
{
    if (app == WEDGE_APP_SSSP && sssp_tiles512(h))
        return SSSP_TILE;
    switch (app) {
    case WEDGE_APP_BFS:
        return 32u * PullEpl<WEDGE_APP_BFS>::value;
    case WEDGE_APP_CC:
        return 32u * PullEpl<WEDGE_APP_CC>::value;
    case WEDGE_APP_SSSP:
        return 32u * PullEpl<WEDGE_APP_SSSP>::value;
    default:
        return 32u * PullEpl<WEDGE_APP_PR>::value;
    }
}

// Size the hub cache of an application's pull, in whole 16-byte lines of the
// gathered array (frontier words for BFS, one property per vertex otherwise):
// the hub-cache knob (0 turns the cache off), within the shared memory a block
// can opt into beside the kernel's static tables.  The cache comes out of the
// SM's L1: on R-MAT scale 24 a 64 KB cache beat both no cache and the largest
// one, whose small L1 left too few gather misses in flight.

static int setup_hub(wedge_graph* h, int app, int precision)
{
    const void* fn = pull_fn(h, app);
    /* the 512-edge SSSP pull runs as two instantiations with one shared-memory layout */
    const void* fn2 = (app == WEDGE_APP_SSSP && sssp_tiles512(h)) ? (const void*)sssp_pull_kernel<true> : nullptr;
    cudaFuncAttributes fa;
    WEDGE_CHECK(cudaFuncGetAttributes(&fa, fn));
    if (fn2) {
        cudaFuncAttributes fb;
        WEDGE_CHECK(cudaFuncGetAttributes(&fb, fn2));
        fa.sharedSizeBytes = fa.sharedSizeBytes > fb.sharedSizeBytes ? fa.sharedSizeBytes : fb.sharedSizeBytes;
    }
    int optin = 0;
    WEDGE_CHECK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
    const uint64_t elem = (app == WEDGE_APP_SSSP) ? (h->s.dist32 ? 4 : 8)
                          : (app == WEDGE_APP_PR && precision != WEDGE_PREC_FP32C) ? 8 : 4;
    const uint64_t stage = (app == WEDGE_APP_SSSP && sssp_tiles512(h)) ? SSSP_STAGE_BYTES : 0u; /* after the cache */
    uint64_t avail = (uint64_t)optin > fa.sharedSizeBytes + stage + 64u ? (uint64_t)optin - fa.sharedSizeBytes - stage - 64u : 0u;
    const uint64_t want = knob_value(h, WEDGE_KNOB_HUB_BYTES);
    if (want < avail)
        avail = want;
    const uint64_t have = (app == WEDGE_APP_BFS) ? (h->g.V + 31) / 32 : h->g.V;
    uint64_t n = avail / elem;
    if (n > have)
        n = have;
    n &= ~3ull;
    h->s.hub_n = (uint32_t)n;
    h->s.hub_tile = 0;
    h->s.hub_k = 0;
    h->hub_bytes = (uint32_t)(n * elem);
    h->s.hub_bytes = h->hub_bytes;
    h->pull_smem = h->hub_bytes + (uint32_t)stage;
    WEDGE_CHECK(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)h->pull_smem));
    if (fn2)
        WEDGE_CHECK(cudaFuncSetAttribute(fn2, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)h->pull_smem));
    if (two_phase_app(app) && n) {
        uint32_t* d = (uint32_t*)(h->s.block_part + h->pull_grid); /* counters: scratch until the first pull */
        hub_split_kernel<<<1, 1, 0, h->stream>>>(h->g, (uint32_t)n, pull_tile_e(h, app), d);
        WEDGE_CHECK(cudaGetLastError());
        uint32_t t[2] = {0, 0};
        WEDGE_CHECK(cudaMemcpyAsync(t, d, sizeof(t), cudaMemcpyDeviceToHost, h->stream));
        WEDGE_CHECK(cudaStreamSynchronize(h->stream));
        h->s.hub_tile = t[0];
        h->s.hub_k = t[1];
    }
    return WEDGE_OK;
}

// dynamic shared memory of pr32_pull_kernel beyond its hub cache: the staged sums
constexpr uint32_t PR32_STAGE_BYTES = (PULL_THREADS / 32) * PR32_SLOTS * sizeof(float);

// hub cache of the compensated-FP32 pull: the hub-cache knob's bytes
// of the rank array, within what the block can opt into beside the staged sums
static int pr32_setup_hub(wedge_graph* h)
{
    cudaFuncAttributes fa;
    WEDGE_CHECK(cudaFuncGetAttributes(&fa, pr32_pull_kernel));
    int optin = 0;
    WEDGE_CHECK(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, h->device));
    const uint64_t fixed = fa.sharedSizeBytes + PR32_STAGE_BYTES + 64u;
    if ((uint64_t)optin < fixed)
        return WEDGE_ERR_UNSUPPORTED;
    uint64_t avail = (uint64_t)optin - fixed;
    const uint64_t want = knob_value(h, WEDGE_KNOB_HUB_BYTES);
    if (want < avail)
        avail = want;
    uint64_t n = avail / 4u;
    if (n > h->g.V)
        n = h->g.V;
    n &= ~3ull; /* whole 16-byte lines */
    h->s.hub_n = (uint32_t)n;
    h->s.hub_bytes = (uint32_t)(n * 4u);
    h->hub_bytes = h->s.hub_bytes;
    WEDGE_CHECK(cudaFuncSetAttribute(pr32_pull_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(h->hub_bytes + PR32_STAGE_BYTES)));
    return WEDGE_OK;
}

// State of the compensated-FP32 PageRank: the double-buffered FP32 ranks,
// FP32 1/outdegree', the split lists of its PR32_TILE-edge tiles, the lists of
// vertices without in-edges, and the per-block sums of the total rank.
static int pr32_state(wedge_graph* h)
{
    DevGraph& g = h->g;
    DevState& s = h->s;
    cudaStream_t st = h->stream;
    const uint64_t V = g.V;
    const uint32_t cap = (uint32_t)h->num_sms * 8u;
    int rc;
    s.rstride = (V + 31) & ~31ull;
    s.pT = (uint32_t)(g.Epad / PR32_TILE);
    if ((rc = dalloc(h, &s.rank32, 2 * s.rstride, true)) || (rc = dalloc(h, &s.inv32, V, true)) ||
        (rc = dalloc(h, &s.pmass, (uint64_t)h->pull_grid + cap + 8, true)) ||
        (rc = dalloc(h, &s.psplit_k, (uint64_t)s.pT + 1, true)) || (rc = dalloc(h, &s.psplit_t0, (uint64_t)s.pT + 1, true)) ||
        (rc = dalloc(h, &s.psplit_t1, (uint64_t)s.pT + 1, true)) || (rc = dalloc(h, &s.phead, (uint64_t)s.pT + 1, true)) ||
        (rc = dalloc(h, &s.ptail, (uint64_t)s.pT + 1, true)))
        return rc;
    pr32_inv_kernel<<<grid_for(V, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(g, s.inv32);
    // destinations spanning the pull's tiles
    unsigned int* d_cnt = nullptr;
    WEDGE_CHECK(cudaMallocAsync((void**)&d_cnt, 2 * sizeof(unsigned int), st));
    WEDGE_CHECK(cudaMemsetAsync(d_cnt, 0, 2 * sizeof(unsigned int), st));
    if (g.Vne)
        split_kernel<<<grid_for(g.Vne, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(g.dst_off, g.Vne, s.pT, PR32_TILE, s.psplit_k,
                                                                               s.psplit_t0, s.psplit_t1, d_cnt);
    unsigned int nsplit[2] = {0, 0};
    WEDGE_CHECK(cudaMemcpyAsync(nsplit, d_cnt, sizeof(nsplit), cudaMemcpyDeviceToHost, st));
    // complete destinations past a tile's staged slots, in tile order
    const uint32_t T = (uint32_t)((g.E + PR32_TILE - 1) / PR32_TILE);
    s.novf = 0;
    if ((rc = dalloc(h, &s.ovf_sum, (uint64_t)g.Vne + 1, true)))
        return rc;
    if (T) {
        uint32_t *cnt = nullptr, *off = nullptr;
        WEDGE_CHECK(cudaMallocAsync((void**)&cnt, T * sizeof(uint32_t), st));
        WEDGE_CHECK(cudaMallocAsync((void**)&off, T * sizeof(uint32_t), st));
        pr32_overflow_kernel<<<grid_for(T, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(g, T, cnt, nullptr, nullptr);
        if ((rc = device_scan(h, cnt, off, T, false)))
            return rc;
        uint32_t last[2] = {0, 0};
        WEDGE_CHECK(cudaMemcpyAsync(&last[0], cnt + (T - 1), 4, cudaMemcpyDeviceToHost, st));
        WEDGE_CHECK(cudaMemcpyAsync(&last[1], off + (T - 1), 4, cudaMemcpyDeviceToHost, st));
        WEDGE_CHECK(cudaStreamSynchronize(st));
        s.novf = last[0] + last[1];
        if ((rc = dalloc(h, &s.ovf_list, (uint64_t)s.novf + 1, true)))
            return rc;
        pr32_overflow_kernel<<<grid_for(T, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(g, T, cnt, off, s.ovf_list);
        cudaFreeAsync(cnt, st);
        cudaFreeAsync(off, st);
    }
    // vertices without in-edges, in id order: with out-edges (gathered, so written every
    // iteration) and without (written once at the end)
    if (V == 0) {
        s.pnsplit = s.pnwide = s.nz = s.ni = 0;
        WEDGE_CHECK(cudaStreamSynchronize(st));
        cudaFree(d_cnt);
        return WEDGE_OK;
    }
    const uint64_t words = (V + 31) / 32;
    uint32_t *has_in = nullptr, *fz = nullptr, *fi = nullptr, *pz = nullptr, *pi = nullptr;
    WEDGE_CHECK(cudaMallocAsync((void**)&has_in, words * sizeof(uint32_t), st));
    WEDGE_CHECK(cudaMallocAsync((void**)&fz, V * sizeof(uint32_t), st));
    WEDGE_CHECK(cudaMallocAsync((void**)&fi, V * sizeof(uint32_t), st));
    WEDGE_CHECK(cudaMallocAsync((void**)&pz, V * sizeof(uint32_t), st));
    WEDGE_CHECK(cudaMallocAsync((void**)&pi, V * sizeof(uint32_t), st));
    WEDGE_CHECK(cudaMemsetAsync(has_in, 0, words * sizeof(uint32_t), st));
    if (g.Vne)
        mark_has_in_kernel<<<grid_for(g.Vne, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(g, has_in);
    pr32_noin_flags_kernel<<<grid_for(V, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(g, has_in, fz, fi);
    if ((rc = device_scan(h, fz, pz, V, false)) || (rc = device_scan(h, fi, pi, V, false)))
        return rc;
    uint32_t tail[4] = {0, 0, 0, 0}; /* last flag and position of each list */
    WEDGE_CHECK(cudaMemcpyAsync(&tail[0], fz + (V - 1), 4, cudaMemcpyDeviceToHost, st));
    WEDGE_CHECK(cudaMemcpyAsync(&tail[1], pz + (V - 1), 4, cudaMemcpyDeviceToHost, st));
    WEDGE_CHECK(cudaMemcpyAsync(&tail[2], fi + (V - 1), 4, cudaMemcpyDeviceToHost, st));
    WEDGE_CHECK(cudaMemcpyAsync(&tail[3], pi + (V - 1), 4, cudaMemcpyDeviceToHost, st));
    WEDGE_CHECK(cudaStreamSynchronize(st));
    s.pnsplit = nsplit[0];
    s.pnwide = nsplit[1];
    s.nz = tail[0] + tail[1];
    s.ni = tail[2] + tail[3];
    if ((rc = dalloc(h, &s.zlist, (uint64_t)s.nz + 1, true)) || (rc = dalloc(h, &s.ilist, (uint64_t)s.ni + 1, true)))
        return rc;
    compact_flags_kernel<<<grid_for(V, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(fz, pz, V, s.zlist);
    compact_flags_kernel<<<grid_for(V, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(fi, pi, V, s.ilist);
    cudaFreeAsync(d_cnt, st);
    cudaFreeAsync(has_in, st);
    cudaFreeAsync(fz, st);
    cudaFreeAsync(fi, st);
    cudaFreeAsync(pz, st);
    cudaFreeAsync(pi, st);
    WEDGE_CHECK(cudaStreamSynchronize(st));
    WEDGE_CHECK(cudaGetLastError());
    return WEDGE_OK;
}

// state arrays of one application (allocated on first use, reused by later runs)
// Split lists of the 512-edge SSSP pull's tiles (destinations spanning tiles:
// short ones from the front, long ones from the back) and their per-tile
// partial minima
static int sssp_split_state(wedge_graph* h)
{
    DevGraph& g = h->g;
    DevState& s = h->s;
    cudaStream_t st = h->stream;
    const uint32_t cap = (uint32_t)h->num_sms * 8u;
    int rc;
    s.pT = (uint32_t)(g.Epad / SSSP_TILE);
    if ((rc = dalloc(h, &s.psplit_k, (uint64_t)s.pT + 1, true)) || (rc = dalloc(h, &s.psplit_t0, (uint64_t)s.pT + 1, true)) ||
        (rc = dalloc(h, &s.psplit_t1, (uint64_t)s.pT + 1, true)) || (rc = dalloc(h, &s.shead, (uint64_t)s.pT + 1, true)) ||
        (rc = dalloc(h, &s.stail, (uint64_t)s.pT + 1, true)))
        return rc;
    unsigned int* d_cnt = nullptr;
    WEDGE_CHECK(cudaMallocAsync((void**)&d_cnt, 2 * sizeof(unsigned int), st));
    WEDGE_CHECK(cudaMemsetAsync(d_cnt, 0, 2 * sizeof(unsigned int), st));
    if (g.Vne)
        split_kernel<<<grid_for(g.Vne, AUX_THREADS, cap), AUX_THREADS, 0, st>>>(g.dst_off, g.Vne, s.pT, SSSP_TILE, s.psplit_k,
                                                                               s.psplit_t0, s.psplit_t1, d_cnt);
    WEDGE_CHECK(cudaGetLastError());
    unsigned int n[2] = {0, 0};
    WEDGE_CHECK(cudaMemcpyAsync(n, d_cnt, sizeof(n), cudaMemcpyDeviceToHost, st));
    WEDGE_CHECK(cudaStreamSynchronize(st));
    cudaFreeAsync(d_cnt, st);
    s.pnsplit = n[0];
    s.pnwide = n[1];
    return WEDGE_OK;
}

static int ensure_state(wedge_graph* h, int app, int precision)
{
    if (h->built_app == app && (app != WEDGE_APP_PR || h->last_precision == precision))
        return WEDGE_OK;
    free_state(h);
    DevGraph& g = h->g;
    DevState& s = h->s;
    const uint64_t V = g.V;
    const uint64_t nwords = (V + 31) / 32 + 1;
    const uint64_t grid = h->pull_grid;
    int rc;
    Ctrl* ctrl;
    double* bp;
    // [grid] block sums | [counter_slots * NCNT] block counters | [aux grid] PageRank-sum partials
    const uint64_t slots = counter_slots(h);
    if ((rc = dalloc(h, &ctrl, 1, true)) ||
        (rc = dalloc(h, &bp, grid + slots * NCNT + (uint64_t)h->num_sms * 8 + 8, true)) ||
        (rc = dalloc(h, &s.log, LOG_CAP, true)))
        return rc;
    WEDGE_CHECK(cudaMemset(ctrl, 0, sizeof(Ctrl)));
    s.ctrl = ctrl;
    s.block_part = bp; /* [grid] doubles, then the counters */
    WEDGE_CHECK(cudaMemset(bp, 0, sizeof(double) * (grid + slots * NCNT)));
    s.app = (uint32_t)app;
    s.push = (app == WEDGE_APP_SSSP && g.csri_pos) ? 1u : 0u;
    s.probe_edges = (uint32_t)knob_value(h, WEDGE_KNOB_PROBE_EDGES);
    if (app == WEDGE_APP_PR && precision == WEDGE_PREC_FP32C) {
        if ((rc = pr32_state(h)))
            return rc;
    } else if (app == WEDGE_APP_PR) {
        if ((rc = dalloc(h, &s.acc, V, true)) || (rc = dalloc(h, &s.inv_od, V, true)))
            return rc;
        pr_inv_outdeg_kernel<<<grid_for(V, AUX_THREADS, (uint32_t)h->num_sms * 8u), AUX_THREADS, 0, h->stream>>>(g, s.inv_od);
        WEDGE_CHECK(cudaGetLastError());
        if ((rc = dalloc(h, &s.rank, V, true)) || (rc = dalloc(h, &s.head_part, (uint64_t)g.T + 1, true)) ||
            (rc = dalloc(h, &s.tail_part, (uint64_t)g.T + 1, true)))
            return rc;
    } else {
        if (app == WEDGE_APP_SSSP) {
            if ((rc = dalloc(h, &s.prop64, V, true)))
                return rc;
            // uint64 weights: the pulls gather a 32-bit copy of the distances
            // (knob WEDGE_KNOB_SSSP_NARROW = 0: the 64-bit distances)
            const uint64_t nk = knob_value(h, WEDGE_KNOB_SSSP_NARROW);
            if (g.weight_kind != WEDGE_WEIGHTS_F64 && nk && (rc = dalloc(h, &s.dist32, V, true)))
                return rc;
            s.narrow_lim = nk > 1u ? (uint32_t)nk : NONE32; /* a limit below 2^32-1 tests the switch to 64 bits */
            s.narrow_sums = g.shard ? 0u : 1u;
            if (sssp_tiles512(h) && (rc = sssp_split_state(h)))
                return rc;
        } else if ((rc = dalloc(h, &s.prop32, V, true))) {
            return rc;
        }
        if ((rc = dalloc(h, &s.front0, nwords, true)) || (rc = dalloc(h, &s.front1, nwords, true)) ||
            (rc = dalloc(h, &s.chunk_bits, (uint64_t)g.T / TILES_PER_WORD + REGION_WORDS + 2, true)) ||
            (rc = dalloc(h, &s.summary, (uint64_t)g.T / TILES_PER_REGION / 32 + 2, true)) ||
            (rc = dalloc(h, &s.tile_list, (uint64_t)g.T + 1, true)) ||
            (rc = dalloc(h, &s.items, V + g.E / PIECE + 2, true)) || (rc = dalloc(h, &s.alist, V + 1, true)))
            return rc;
        if (app == WEDGE_APP_BFS || app == WEDGE_APP_CC) {
            if ((rc = dalloc(h, &s.vis_c, (uint64_t)g.Vne / 32 + 2, true)))
                return rc;
        }
        if (app == WEDGE_APP_CC && g.sym) {
            if ((rc = dalloc(h, &s.cc_best, V, true)))
                return rc;
        }
        if (app == WEDGE_APP_BFS || app == WEDGE_APP_CC) {
            if ((rc = dalloc(h, &s.tile_open, (uint64_t)g.T / 32 + 2, true)))
                return rc;
        }
        if (app == WEDGE_APP_BFS || app == WEDGE_APP_CC) {
            if ((rc = dalloc(h, &s.tile_need, (uint64_t)g.T / 32 + 2, true)))
                return rc;
        }
        if ((app == WEDGE_APP_BFS || app == WEDGE_APP_CC) && g.csri_pos) { /* Wedge pulls over candidate destinations */
            if ((rc = dalloc(h, &s.cand, (uint64_t)g.Vne / 32 + 2, true)) ||
                (rc = dalloc(h, &s.cand_list, (uint64_t)g.Vne + 1, true)))
                return rc;
        }
    }
    if ((rc = (app == WEDGE_APP_PR && precision == WEDGE_PREC_FP32C) ? pr32_setup_hub(h) : setup_hub(h, app, precision)))
        return rc;
    h->built_app = app;
    h->last_precision = precision;
    return WEDGE_OK;
}

static unsigned long long* counters(wedge_graph* h) { return (unsigned long long*)(h->s.block_part + h->pull_grid); }

// counter slots the pulls of one iteration fill (two launches for CC/SSSP)
static uint32_t pull_slots(wedge_graph* h, int app)
{
    return h->dst_grid * dst_launches_of(app) + h->pull_grid * (pull_launches_of(app) - dst_launches_of(app));
}

// PageRank-sum partials after the counters
static double* pr_sums(wedge_graph* h) { return (double*)(counters(h) + counter_slots(h) * NCNT); }

template <int APP>
static void launch_pull_app(wedge_graph* h)
{
    constexpr int EPL = PullEpl<APP>::value;
    const uint32_t grid = h->pull_grid;
    unsigned long long* cnt = counters(h);
    if constexpr (APP == WEDGE_APP_BFS || APP == WEDGE_APP_CC) {
        const uint32_t dgrid = h->dst_grid;
        dst_kernel<APP, EPL><<<dgrid, PULL_THREADS, 0, h->stream>>>(h->g, h->s, cnt, PHASE_DST_A);
        cnt += (uint64_t)NCNT * dgrid;
        if (APP == WEDGE_APP_CC) {
            dst_kernel<APP, EPL><<<dgrid, PULL_THREADS, 0, h->stream>>>(h->g, h->s, cnt, PHASE_DST_B);
            cnt += (uint64_t)NCNT * dgrid;
        }
    }
    if (APP == WEDGE_APP_SSSP && sssp_tiles512(h)) {
        const uint32_t sgrid = sssp_split_grid(h);
        sssp_pull_kernel<false><<<grid, PULL_THREADS, h->pull_smem, h->stream>>>(h->g, h->s, cnt, PHASE_HUBS);
        sssp_pull_kernel<true><<<grid, PULL_THREADS, h->pull_smem, h->stream>>>(h->g, h->s, cnt, PHASE_HUBS);
        sssp_split_kernel<<<sgrid, AUX_THREADS, 0, h->stream>>>(h->g, h->s, cnt, grid, PHASE_HUBS);
        sssp_pull_kernel<false><<<grid, PULL_THREADS, h->pull_smem, h->stream>>>(h->g, h->s, cnt + NCNT * grid,
                                                                                 PHASE_REST);
        sssp_pull_kernel<true><<<grid, PULL_THREADS, h->pull_smem, h->stream>>>(h->g, h->s, cnt + NCNT * grid,
                                                                                PHASE_REST);
        sssp_split_kernel<<<sgrid, AUX_THREADS, 0, h->stream>>>(h->g, h->s, cnt + NCNT * grid, grid, PHASE_REST);
    } else if (two_phase_app(APP)) {
        pull_kernel<APP, EPL><<<grid, PULL_THREADS, h->hub_bytes, h->stream>>>(h->g, h->s, cnt, PHASE_HUBS);
        pull_kernel<APP, EPL><<<grid, PULL_THREADS, h->hub_bytes, h->stream>>>(h->g, h->s, cnt + NCNT * grid,
                                                                               PHASE_REST);
    } else {
        pull_kernel<APP, EPL><<<grid, PULL_THREADS, h->hub_bytes, h->stream>>>(h->g, h->s, cnt, PHASE_ALL);
    }
}

static void launch_pull(wedge_graph* h, int app)
{
    switch (app) {
    case WEDGE_APP_BFS:
        launch_pull_app<WEDGE_APP_BFS>(h);
        break;
    case WEDGE_APP_CC:
        launch_pull_app<WEDGE_APP_CC>(h);
        break;
    case WEDGE_APP_SSSP:
        launch_pull_app<WEDGE_APP_SSSP>(h);
        break;
    default:
        launch_pull_app<WEDGE_APP_PR>(h);
        break;
    }
}

// kernels one iteration launches: the pull(s) and the five of the tail
// the Wedge build's launches: collect, expand, build (not for SSSP over
// in-edge positions), compact (chunk frontiers only)
static uint64_t build_launches(const wedge_graph* h)
{
    return 2ull + (h->s.push ? 0ull : 1ull) + ((h->s.cand || h->s.push) ? 0ull : 1ull);
}

static uint64_t iteration_launches(const wedge_graph* h, int app)
{
    /* decide, the build, the pull (the 512-edge SSSP pull: two instantiations per launch and a
       split-destination finish after each) */
    const uint64_t pulls = pull_launches_of(app) * ((app == WEDGE_APP_SSSP && sssp_tiles512(h)) ? 3ull : 1ull);
    return 1ull + build_launches(h) + pulls;
}

// sssp_split_kernel: a thread per short split, a warp per long one
static uint32_t sssp_split_grid(wedge_graph* h)
{
    const uint64_t wide = (uint64_t)h->s.pnwide * 32u;
    return grid_for((h->s.pnsplit > wide ? h->s.pnsplit : wide) + 1, AUX_THREADS, (uint32_t)h->num_sms * 8u);
}

static uint32_t aux_grid(wedge_graph* h, uint64_t work)
{
    return grid_for(work, AUX_THREADS, (uint32_t)h->num_sms * 8u);
}

// PageRank total rank into Ctrl::pr_total; its block sums use the PageRank-sum
// partials (num_sms * 8 + 8 doubles after the counters)
static void launch_pr_total(wedge_graph* h)
{
    pr_total_kernel<<<aux_grid(h, h->g.V), AUX_THREADS, 0, h->stream>>>(h->s.acc, h->g.V, pr_sums(h), h->s.ctrl);
}

// PageRank merge: a thread per short split, a warp per long one
static uint32_t finish_grid(wedge_graph* h, const DevGraph& g)
{
    const uint64_t wide = (uint64_t)g.nwide * 32u;
    return aux_grid(h, (g.nsplit > wide ? g.nsplit : wide) + 1);
}

// Wedge frontier -> tile list, with the tile size of the application's pull
static void launch_compact(wedge_graph* h, int app)
{
    const uint64_t regions = ((uint64_t)h->g.T / TILES_PER_WORD + REGION_WORDS) / REGION_WORDS;
    const uint32_t grid = aux_grid(h, regions * 32);
    if (app == WEDGE_APP_BFS)
        compact_kernel<PullEpl<WEDGE_APP_BFS>::value><<<grid, AUX_THREADS, 0, h->stream>>>(h->g, h->s);
    else if (app == WEDGE_APP_CC)
        compact_kernel<PullEpl<WEDGE_APP_CC>::value><<<grid, AUX_THREADS, 0, h->stream>>>(h->g, h->s);
    else
        compact_kernel<PullEpl<WEDGE_APP_SSSP>::value><<<grid, AUX_THREADS, 0, h->stream>>>(h->g, h->s);
}

// Wedge frontier of the next pull (no-ops unless it is a Wedge pull)
static void launch_wedge_build(wedge_graph* h, const DevGraph& g, int app)
{
    collect_kernel<<<aux_grid(h, (g.V + 31) / 32), AUX_THREADS, 0, h->stream>>>(g, h->s, (uint32_t)app);
    expand_kernel<<<h->build_grid, AUX_THREADS, 0, h->stream>>>(g, h->s);
    if (!h->s.push) /* SSSP over in-edge positions: the pull takes expand_kernel's items */
        wedge_build_kernel<<<h->build_grid, AUX_THREADS, 0, h->stream>>>(g, h->s);
    if (!h->s.cand && !h->s.push) /* over in-edge positions the build lists candidates or items, not tiles */
        launch_compact(h, app);
}

// iteration tail after a pull: mass/convergence, Wedge frontier, bitmap reset
static void launch_tail(wedge_graph* h, int app)
{
    decide_kernel<<<1, AUX_THREADS, 0, h->stream>>>(h->g, h->s, counters(h), pull_slots(h, app), (uint32_t)app);
    launch_wedge_build(h, h->g, app); /* collect_kernel clears the bitmaps for the next pull */
}

static void launch_init(wedge_graph* h, int app, uint64_t root, uint32_t sched, unsigned long long thr, uint32_t max_iter,
                        uint32_t probe_iter = 0xFFFFFFFFu, uint32_t probe_mode = MODE_DENSE)
{
    const uint64_t work = h->g.V > h->g.T ? h->g.V : h->g.T;
    const uint32_t tile_e = pull_tile_e(h, app);
    const uint32_t topen = (uint32_t)((h->g.E + tile_e - 1) / tile_e); /* pull tiles holding in-edges */
    init_kernel<<<aux_grid(h, work), AUX_THREADS, 0, h->stream>>>(h->g, h->s, (uint32_t)app, topen);
    init_root_kernel<<<1, 32, 0, h->stream>>>(h->g, h->s, (uint32_t)app, root, sched, thr,
                                                                           max_iter, probe_iter, probe_mode);
    h->cc_pending = (app == WEDGE_APP_CC && h->s.cc_best) ? 1 : 0;
    launch_wedge_build(h, h->g, app); /* collect_kernel clears the bitmaps for the first pull */
}

// CC on a symmetric graph, once the labels converged: caller-id labels in
// place (2 launches; best was preset by init_kernel)
static void cc_finalize(wedge_graph* h)
{
    cc_best_kernel<<<aux_grid(h, h->g.V), AUX_THREADS, 0, h->stream>>>(h->g, h->s.prop32, h->s.cc_best);
    cc_apply_kernel<<<aux_grid(h, h->g.V), AUX_THREADS, 0, h->stream>>>(h->g, h->s.prop32, h->s.cc_best);
    h->cc_pending = 0;
}

// The state the results are read from: while CC labels are engine ids (a
// traversal driven phase by phase), a lookup table of the caller-id labels is
// built beside them, leaving the labels themselves for further pulls.
static int result_state(wedge_graph* h, DevState* out)
{
    *out = h->s;
    if (h->last_app == WEDGE_APP_CC && h->cc_pending) {
        WEDGE_CHECK(cudaMemsetAsync(h->s.cc_best, 0xFF, h->g.V * sizeof(uint32_t), h->stream));
        cc_best_kernel<<<aux_grid(h, h->g.V), AUX_THREADS, 0, h->stream>>>(h->g, h->s.prop32, h->s.cc_best);
        out->cc_map = h->s.cc_best;
    }
    return WEDGE_OK;
}

static int read_ctrl(wedge_graph* h, Ctrl* out)
{
    WEDGE_CHECK(cudaMemcpyAsync(h->h_ctrl, h->s.ctrl, sizeof(Ctrl), cudaMemcpyDeviceToHost, h->stream));
    WEDGE_CHECK(cudaStreamSynchronize(h->stream));
    memcpy(out, h->h_ctrl, sizeof(Ctrl));
    return WEDGE_OK;
}

// Captures one iteration (pull + tail) as the body of a device-side while
// loop; the loop condition is Ctrl::loop, set by decide_kernel through
// loop_cond_kernel.
__global__ void loop_cond_kernel(DevState s, cudaGraphConditionalHandle handle)
{
    cudaGraphSetConditional(handle, s.ctrl->loop);
}

static int build_graph(wedge_graph* h, int app)
{
    if (h->graph_exec && h->graph_app == app)
        return WEDGE_OK;
    if (h->graph_exec) {
        cudaGraphExecDestroy(h->graph_exec);
        h->graph_exec = nullptr;
    }
    cudaGraph_t graph;
    WEDGE_CHECK(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle handle;
    WEDGE_CHECK(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cparams = {};
    cparams.type = cudaGraphNodeTypeConditional;
    cparams.conditional.handle = handle;
    cparams.conditional.type = cudaGraphCondTypeWhile;
    cparams.conditional.size = 1;
    cudaGraphNode_t cnode;
    WEDGE_CHECK(cudaGraphAddNode(&cnode, graph, nullptr, nullptr, 0, &cparams));
    cudaGraph_t body = cparams.conditional.phGraph_out[0];
    // captured on the handle's own stream (a caller's stream may carry other work)
    const cudaStream_t run_stream = h->stream;
    h->stream = h->own_stream;
    WEDGE_CHECK(cudaStreamBeginCaptureToGraph(h->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    launch_pull(h, app);
    launch_tail(h, app);
    loop_cond_kernel<<<1, 1, 0, h->stream>>>(h->s, handle);
    cudaGraph_t captured;
    const cudaError_t ce = cudaStreamEndCapture(h->stream, &captured);
    h->stream = run_stream;
    WEDGE_CHECK(ce);
    WEDGE_CHECK(cudaGraphInstantiate(&h->graph_exec, graph, 0));
    cudaGraphDestroy(graph);
    h->graph_app = app;
    return WEDGE_OK;
}

// The statistics of the traversal that just ran on h->stream (waits for it).
// launches: the kernels launched from the host; a graph loop adds its
// iterations' launches and the loop condition's.
static int traversal_stats(wedge_graph* h, int app, uint64_t launches, bool use_graph, bool timing, double t_pull_dense,
                           double t_pull_wedge, double t_wedge, wedge_stats_t* st)
{
    Ctrl c;
    int rc = read_ctrl(h, &c);
    if (rc)
        return rc;
    float total = 0;
    cudaEventElapsedTime(&total, h->ev[0], h->ev[1]);
    h->last_app = app;
    h->last_timing = timing;
    if (st) {
        memset(st, 0, sizeof(*st));
        st->dsts_scanned = c.dsts_scanned;
        st->vertices_activated = c.activated;
        st->iterations = c.iter;
        st->wedge_iterations = c.wedge_iters;
        st->running_ms = total;
        st->pull_ms_dense = t_pull_dense;
        st->pull_ms_wedge = t_pull_wedge;
        st->wedge_ms = t_wedge;
        st->edges_scanned = c.edges_scanned;
        st->tiles_scanned = c.tiles_scanned;
        st->pull_launches = c.pull_launches;
        st->kernel_launches = use_graph ? launches + (iteration_launches(h, app) + 1ull) * c.iter : launches;
    }
    if (c.error)
        return WEDGE_ERR_CUDA;
    if (c.not_converged)
        return WEDGE_ERR_NOT_CONVERGED;
    return WEDGE_OK;
}

// One traversal.  With wait false (graph loop only) the work is queued and the
// statistics are left to traversal_stats, through wedge_cuda_wait.
static int run_traversal(wedge_graph* h, int app, const wedge_params_t* p, wedge_stats_t* st, bool wait = true)
{
    const DevGraph& g = h->g;
    const uint64_t root = p->root < g.V ? p->root : 0; /* main.c:81-85 */
    const unsigned long long thr = (unsigned long long)((g.E_thr * (unsigned long long)p->threshold_pct) / 100ull);
    uint64_t cap = p->max_iterations ? p->max_iterations : g.V + 1;
    if (cap > 0x7fffffffull)
        cap = 0x7fffffffull;
    const bool timing = (p->flags & WEDGE_FLAG_TIMING) != 0;
    const bool use_graph = (p->flags & WEDGE_FLAG_GRAPH) != 0 && !timing;
    uint64_t launches = 0;
    double t_pull_dense = 0, t_pull_wedge = 0, t_wedge = 0;
    if (use_graph) {
        int rc = build_graph(h, app);
        if (rc)
            return rc;
    }
    WEDGE_CHECK(cudaEventRecord(h->ev[0], h->stream));
    launch_init(h, app, root, (uint32_t)p->sched, thr, (uint32_t)cap, p->probe_iter, (uint32_t)p->probe_mode);
    launches += 2ull + build_launches(h); /* init, root, the Wedge build */
    Ctrl c;
    if (use_graph) {
        WEDGE_CHECK(cudaGraphLaunch(h->graph_exec, h->stream));
    } else if (timing) {
        for (;;) {
            int rc = read_ctrl(h, &c);
            if (rc)
                return rc;
            if (c.done)
                break;
            const uint32_t mode = c.mode;
            WEDGE_CHECK(cudaEventRecord(h->ev[2], h->stream));
            launch_pull(h, app);
            WEDGE_CHECK(cudaEventRecord(h->ev[3], h->stream));
            launch_tail(h, app);
            WEDGE_CHECK(cudaEventRecord(h->ev[4], h->stream));
            launches += iteration_launches(h, app);
            WEDGE_CHECK(cudaEventSynchronize(h->ev[4]));
            float a = 0, b = 0;
            cudaEventElapsedTime(&a, h->ev[2], h->ev[3]);
            cudaEventElapsedTime(&b, h->ev[3], h->ev[4]);
            if (mode != MODE_WEDGE)
                t_pull_dense += a;
            else
                t_pull_wedge += a;
            t_wedge += b;
            if (c.iter < LOG_CAP) {
                h->iter_pull_ms[c.iter] = a;
                h->iter_wedge_ms[c.iter] = b;
            }
        }
    } else {
        // speculative batches: kernels are no-ops once Ctrl::done is set
        for (;;) {
            for (int b = 0; b < 3; ++b) {
                launch_pull(h, app);
                launch_tail(h, app);
                launches += iteration_launches(h, app);
            }
            int rc = read_ctrl(h, &c);
            if (rc)
                return rc;
            if (c.done)
                break;
        }
    }
    if (app == WEDGE_APP_CC && h->cc_pending) {
        cc_finalize(h);
        launches += 2;
    }
    WEDGE_CHECK(cudaEventRecord(h->ev[1], h->stream));
    WEDGE_CHECK(cudaGetLastError());
    h->last_app = app;
    if (!wait && use_graph) {
        h->pend_app = app;
        h->pend_launches = launches;
        return WEDGE_OK;
    }
    return traversal_stats(h, app, launches, use_graph, timing, t_pull_dense, t_pull_wedge, t_wedge, st);
}

// compensated-FP32 PageRank: the grid of pr32_finish_kernel (a thread per short
// split and per vertex without in-edges, a warp per long split)
static uint32_t pr32_finish_grid(wedge_graph* h)
{
    const DevState& s = h->s;
    uint64_t work = (uint64_t)s.pnwide * 32u;
    if (s.pnsplit > work)
        work = s.pnsplit;
    if (s.nz > work)
        work = s.nz;
    if (s.novf > work)
        work = s.novf;
    return aux_grid(h, work + 1);
}

// one compensated-FP32 PageRank iteration: pull (with the vertex phase of the
// destinations inside one tile), split destinations, total rank
static void launch_pr32_iteration(wedge_graph* h)
{
    const uint32_t fgrid = pr32_finish_grid(h);
    pr32_pull_kernel<<<h->pull_grid, PULL_THREADS, h->hub_bytes + PR32_STAGE_BYTES, h->stream>>>(h->g, h->s, counters(h));
    pr32_finish_kernel<<<fgrid, AUX_THREADS, 0, h->stream>>>(h->g, h->s, h->pull_grid);
    pr32_total_kernel<<<1, AUX_THREADS, 0, h->stream>>>(h->s, h->pull_grid + fgrid, counters(h), h->pull_grid);
}

// execution_initialize_pr for the compensated-FP32 form: ranks 1/N and the total of iteration 0
static void launch_pr32_init(wedge_graph* h, uint32_t max_iter)
{
    const uint32_t vgrid = aux_grid(h, h->g.V);
    pr32_init_kernel<<<vgrid, AUX_THREADS, 0, h->stream>>>(h->g, h->s, max_iter);
    pr32_total_kernel<<<1, AUX_THREADS, 0, h->stream>>>(h->s, vgrid, nullptr, 0);
}

static void launch_pr32_iso(wedge_graph* h)
{
    pr32_iso_kernel<<<aux_grid(h, h->s.ni), AUX_THREADS, 0, h->stream>>>(h->g, h->s);
}

// Captures one PageRank iteration (pull, ordered merge, vertex phase) as the
// body of a device-side while loop on Ctrl::iter < Ctrl::max_iter.  The
// kernels hold the state by value, so the capture is keyed on the damping
// factor (the precision is part of the state, whose rebuild drops it).
static int build_pr_graph(wedge_graph* h)
{
    uint64_t key;
    memcpy(&key, &h->s.damping, sizeof(key));
    if (h->pr_exec && h->pr_key == key)
        return WEDGE_OK;
    if (h->pr_exec) {
        cudaGraphExecDestroy(h->pr_exec);
        h->pr_exec = nullptr;
    }
    const DevGraph& g = h->g;
    cudaGraph_t graph;
    WEDGE_CHECK(cudaGraphCreate(&graph, 0));
    cudaGraphConditionalHandle handle;
    WEDGE_CHECK(cudaGraphConditionalHandleCreate(&handle, graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cparams = {};
    cparams.type = cudaGraphNodeTypeConditional;
    cparams.conditional.handle = handle;
    cparams.conditional.type = cudaGraphCondTypeWhile;
    cparams.conditional.size = 1;
    cudaGraphNode_t cnode;
    WEDGE_CHECK(cudaGraphAddNode(&cnode, graph, nullptr, nullptr, 0, &cparams));
    cudaGraph_t body = cparams.conditional.phGraph_out[0];
    const cudaStream_t run_stream = h->stream; /* captured on the handle's own stream */
    h->stream = h->own_stream;
    WEDGE_CHECK(cudaStreamBeginCaptureToGraph(h->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed));
    if (h->s.precision == WEDGE_PREC_FP32C) {
        launch_pr32_iteration(h);
    } else {
        launch_pull(h, WEDGE_APP_PR);
        pr_finish_kernel<<<finish_grid(h, g), AUX_THREADS, 0, h->stream>>>(g, h->s, h->pull_grid, counters(h));
        launch_pr_total(h);
        pr_vertex_kernel<<<aux_grid(h, g.V), AUX_THREADS, 0, h->stream>>>(g, h->s);
    }
    pr_loop_cond_kernel<<<1, 1, 0, h->stream>>>(h->s, handle);
    cudaGraph_t captured;
    const cudaError_t ce = cudaStreamEndCapture(h->stream, &captured);
    h->stream = run_stream;
    WEDGE_CHECK(ce);
    WEDGE_CHECK(cudaGraphInstantiate(&h->pr_exec, graph, 0));
    cudaGraphDestroy(graph);
    h->pr_key = key;
    return WEDGE_OK;
}

// The statistics of the PageRank run that just ran on h->stream (waits for it)
static int pr_stats(wedge_graph* h, uint32_t iters, bool use_graph, bool timing, double t_pull, double t_vertex,
                    wedge_stats_t* st)
{
    Ctrl c;
    int rc = read_ctrl(h, &c);
    if (rc)
        return rc;
    float total = 0;
    cudaEventElapsedTime(&total, h->ev[0], h->ev[1]);
    h->last_app = WEDGE_APP_PR;
    h->last_timing = timing;
    const bool c32 = h->s.precision == WEDGE_PREC_FP32C;
    if (st) {
        memset(st, 0, sizeof(*st));
        st->dsts_scanned = c.dsts_scanned;
        st->iterations = iters;
        st->running_ms = total;
        st->pull_ms_dense = t_pull;
        st->vertex_ms = t_vertex;
        st->edges_scanned = c.edges_scanned;
        st->tiles_scanned = c.tiles_scanned;
        st->pull_launches = c.pull_launches;
        /* init (+ total), the iterations (+ the loop condition), the sums (+ isolated vertices) */
        st->kernel_launches = c32 ? 5ull + (use_graph ? 4ull : 3ull) * iters : 3ull + (use_graph ? 5ull : 4ull) * iters;
        st->pr_sum = c.pr_sum;
    }
    if (c.error)
        return WEDGE_ERR_CUDA;
    return WEDGE_OK;
}

static int run_pr(wedge_graph* h, const wedge_params_t* p, wedge_stats_t* st, bool wait = true)
{
    const DevGraph& g = h->g;
    const bool timing = (p->flags & WEDGE_FLAG_TIMING) != 0;
    h->s.damping = p->damping > 0.0 ? p->damping : 0.875;
    h->s.precision = (uint32_t)p->precision;
    const uint32_t vgrid = aux_grid(h, g.V);
    const uint32_t fgrid = finish_grid(h, g);
    const bool use_graph = (p->flags & WEDGE_FLAG_GRAPH) != 0 && !timing && p->num_iterations > 0;
    if (use_graph) {
        int rc = build_pr_graph(h);
        if (rc)
            return rc;
    }
    const bool c32 = h->s.precision == WEDGE_PREC_FP32C;
    double t_pull = 0, t_vertex = 0;
    WEDGE_CHECK(cudaEventRecord(h->ev[0], h->stream));
    if (c32)
        launch_pr32_init(h, p->num_iterations);
    else
        pr_init_kernel<<<vgrid, AUX_THREADS, 0, h->stream>>>(g, h->s, p->num_iterations);
    if (use_graph)
        WEDGE_CHECK(cudaGraphLaunch(h->pr_exec, h->stream));
    for (uint32_t it = 0; !use_graph && it < p->num_iterations; ++it) {
        if (timing)
            WEDGE_CHECK(cudaEventRecord(h->ev[2], h->stream));
        if (c32)
            pr32_pull_kernel<<<h->pull_grid, PULL_THREADS, h->hub_bytes + PR32_STAGE_BYTES, h->stream>>>(g, h->s,
                                                                                                    counters(h));
        else
            launch_pull(h, WEDGE_APP_PR);
        if (timing)
            WEDGE_CHECK(cudaEventRecord(h->ev[3], h->stream));
        if (c32) {
            const uint32_t g32 = pr32_finish_grid(h);
            pr32_finish_kernel<<<g32, AUX_THREADS, 0, h->stream>>>(g, h->s, h->pull_grid);
            pr32_total_kernel<<<1, AUX_THREADS, 0, h->stream>>>(h->s, h->pull_grid + g32, counters(h), h->pull_grid);
        } else {
            pr_finish_kernel<<<fgrid, AUX_THREADS, 0, h->stream>>>(g, h->s, h->pull_grid, counters(h));
            launch_pr_total(h);
            pr_vertex_kernel<<<vgrid, AUX_THREADS, 0, h->stream>>>(g, h->s);
        }
        if (timing) {
            WEDGE_CHECK(cudaEventRecord(h->ev[4], h->stream));
            WEDGE_CHECK(cudaEventSynchronize(h->ev[4]));
            float a = 0, b = 0;
            cudaEventElapsedTime(&a, h->ev[2], h->ev[3]);
            cudaEventElapsedTime(&b, h->ev[3], h->ev[4]);
            t_pull += a;
            t_vertex += b;
            if (it < LOG_CAP) {
                h->iter_pull_ms[it] = a;
                h->iter_wedge_ms[it] = 0.0;
            }
        }
    }
    if (c32)
        launch_pr32_iso(h); /* vertices with neither in- nor out-edges, once */
    WEDGE_CHECK(cudaEventRecord(h->ev[1], h->stream));
    double* sums = pr_sums(h);
    pr_sum_kernel<<<vgrid, AUX_THREADS, 0, h->stream>>>(g, h->s, sums);
    pr_sum_final_kernel<<<1, 32, 0, h->stream>>>(h->s, sums, vgrid);
    WEDGE_CHECK(cudaGetLastError());
    h->last_app = WEDGE_APP_PR;
    if (!wait && !timing) {
        h->pend_app = WEDGE_APP_PR;
        h->pend_iters = p->num_iterations;
        h->pend_launches = use_graph ? 1u : 0u; /* the launch count formula's graph term */
        return WEDGE_OK;
    }
    return pr_stats(h, p->num_iterations, use_graph, timing, t_pull, t_vertex, st);
}

}  // namespace wedge

using namespace wedge;

extern "C" {

int wedge_cuda_abi_version(void) { return WEDGE_CUDA_ABI_VERSION; }

const char* wedge_cuda_status_string(int status)
{
    switch (status) {
    case WEDGE_OK:
        return "ok";
    case WEDGE_ERR_IO:
        return "I/O error";
    case WEDGE_ERR_FORMAT:
        return "malformed graph input";
    case WEDGE_ERR_OOM:
        return "out of memory";
    case WEDGE_ERR_CUDA:
        return "CUDA error";
    case WEDGE_ERR_NOT_CONVERGED:
        return "iteration cap reached before convergence";
    case WEDGE_ERR_ARG:
        return "invalid argument";
    case WEDGE_ERR_UNSUPPORTED:
        return "unsupported";
    default:
        return "unknown status";
    }
}

static int check_params(const wedge_graph_t* g, int app, const wedge_params_t* p)
{
    if (!g || !p || app < WEDGE_APP_BFS || app > WEDGE_APP_SSSP)
        return WEDGE_ERR_ARG;
    if (p->threshold_pct > 100 || p->sched < WEDGE_SCHED_PLAIN || p->sched > WEDGE_SCHED_PROBE)
        return WEDGE_ERR_ARG;
    if (p->sched == WEDGE_SCHED_PROBE && (p->probe_mode < WEDGE_MODE_DENSE || p->probe_mode > WEDGE_MODE_FILTERED))
        return WEDGE_ERR_ARG;
    if (app == WEDGE_APP_PR && (p->precision != WEDGE_PREC_FP64 && p->precision != WEDGE_PREC_FP32C))
        return WEDGE_ERR_ARG;
    if (app == WEDGE_APP_SSSP && g->weight_kind == WEDGE_WEIGHTS_NONE)
        return WEDGE_ERR_ARG; /* SSSP needs a weighted load (application.c:171) */
    return WEDGE_OK;
}

// work on the handle's stream that overwrites state waits for queued asynchronous exports
static int after_exports(wedge_graph_t* g)
{
    if (g->x_pending)
        WEDGE_CHECK(cudaStreamWaitEvent(g->stream, g->ev_x, 0));
    return WEDGE_OK;
}

int wedge_cuda_run(wedge_graph_t* g, int app, const wedge_params_t* params, wedge_stats_t* stats)
{
    int rc = check_params(g, app, params);
    if (rc)
        return rc;
    WEDGE_CHECK(cudaSetDevice(g->device));
    if ((rc = after_exports(g)))
        return rc;
    if ((rc = ensure_state(g, app, params->precision)))
        return rc;
    g->pend_app = -1;
    if (app == WEDGE_APP_PR)
        return run_pr(g, params, stats);
    return run_traversal(g, app, params, stats);
}

int wedge_cuda_run_async(wedge_graph_t* g, int app, const wedge_params_t* params)
{
    int rc = check_params(g, app, params);
    if (rc)
        return rc;
    if (params->flags & WEDGE_FLAG_TIMING)
        return WEDGE_ERR_ARG; /* per-iteration events need the host between iterations */
    WEDGE_CHECK(cudaSetDevice(g->device));
    if ((rc = after_exports(g)))
        return rc;
    if ((rc = ensure_state(g, app, params->precision)))
        return rc;
    wedge_params_t p = *params;
    p.flags |= WEDGE_FLAG_GRAPH; /* the iteration loop runs on the device */
    g->pend_app = -1;
    return app == WEDGE_APP_PR ? run_pr(g, &p, nullptr, false) : run_traversal(g, app, &p, nullptr, false);
}

int wedge_cuda_read_results_async(wedge_graph_t* g, void* host_props, uint64_t bytes)
{
    if (!g || !host_props || bytes < 8ull * g->g.V || g->last_app < 0)
        return WEDGE_ERR_ARG;
    WEDGE_CHECK(cudaSetDevice(g->device));
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, host_props) != cudaSuccess || pa.type != cudaMemoryTypeHost || !pa.devicePointer ||
        ((uintptr_t)pa.devicePointer & 7u) != 0u) {
        cudaGetLastError();
        return WEDGE_ERR_ARG; /* asynchronous reads need page-locked host memory */
    }
    if (!g->xstream)
        WEDGE_CHECK(cudaStreamCreateWithFlags(&g->xstream, cudaStreamNonBlocking));
    if (!g->xbuf) { /* the words are staged in device memory and copied by the copy engine, off the SMs */
        void* p = nullptr;
        WEDGE_CHECK(cudaMalloc(&p, 8ull * (g->g.V ? g->g.V : 1)));
        g->xbuf = (unsigned long long*)p;
    }
    DevState rs;
    int rc = result_state(g, &rs);
    if (rc)
        return rc;
    WEDGE_CHECK(cudaEventRecord(g->ev_run, g->stream));
    WEDGE_CHECK(cudaStreamWaitEvent(g->xstream, g->ev_run, 0));
    export_kernel<<<aux_grid(g, g->g.V), AUX_THREADS, 0, g->xstream>>>(g->g, rs, (uint32_t)g->last_app, g->xbuf);
    WEDGE_CHECK(cudaGetLastError());
    WEDGE_CHECK(cudaMemcpyAsync(host_props, g->xbuf, 8ull * g->g.V, cudaMemcpyDeviceToHost, g->xstream));
    WEDGE_CHECK(cudaEventRecord(g->ev_x, g->xstream));
    g->x_pending = 1;
    return WEDGE_OK;
}

int wedge_cuda_wait(wedge_graph_t* g, wedge_stats_t* stats)
{
    if (!g)
        return WEDGE_ERR_ARG;
    WEDGE_CHECK(cudaSetDevice(g->device));
    WEDGE_CHECK(cudaStreamSynchronize(g->stream));
    if (g->x_pending) {
        WEDGE_CHECK(cudaStreamSynchronize(g->xstream));
        g->x_pending = 0;
    }
    int rc = WEDGE_OK;
    if (g->pend_app == WEDGE_APP_PR)
        rc = pr_stats(g, g->pend_iters, g->pend_launches != 0, false, 0.0, 0.0, stats);
    else if (g->pend_app >= 0)
        rc = traversal_stats(g, g->pend_app, g->pend_launches, true, false, 0.0, 0.0, 0.0, stats);
    else if (stats)
        memset(stats, 0, sizeof(*stats));
    g->pend_app = -1;
    return rc;
}

int wedge_cuda_wait_results(wedge_graph_t* g)
{
    if (!g)
        return WEDGE_ERR_ARG;
    WEDGE_CHECK(cudaSetDevice(g->device));
    if (g->x_pending) {
        WEDGE_CHECK(cudaEventSynchronize(g->ev_x));
        g->x_pending = 0;
    }
    return WEDGE_OK;
}

int wedge_cuda_set_stream(wedge_graph_t* g, void* stream)
{
    if (!g)
        return WEDGE_ERR_ARG;
    WEDGE_CHECK(cudaSetDevice(g->device));
    WEDGE_CHECK(cudaStreamSynchronize(g->stream)); /* the handle's queued work finishes on its old stream */
    g->stream = stream ? (cudaStream_t)stream : g->own_stream;
    return WEDGE_OK;
}

int wedge_cuda_set_knob(wedge_graph_t* g, int knob, uint64_t value)
{
    if (!g || knob < 0 || knob >= WEDGE_KNOBS || (value != WEDGE_KNOB_DEFAULT && !knob_ok(knob, value)))
        return WEDGE_ERR_ARG;
    WEDGE_CHECK(cudaSetDevice(g->device));
    if (g->knob[knob] == value)
        return WEDGE_OK;
    WEDGE_CHECK(cudaStreamSynchronize(g->stream)); /* no queued work may use the state released here */
    if (g->xstream)
        WEDGE_CHECK(cudaStreamSynchronize(g->xstream));
    g->x_pending = 0;
    g->knob[knob] = value;
    free_state(g);
    g->last_app = -1;
    return WEDGE_OK;
}

int wedge_cuda_get_knob(wedge_graph_t* g, int knob, uint64_t* value)
{
    if (!g || !value || knob < 0 || knob >= WEDGE_KNOBS)
        return WEDGE_ERR_ARG;
    *value = knob_value(g, knob);
    return WEDGE_OK;
}

/* ------------------------------------------------------------ shards */

}  // extern "C"

namespace wedge {
// the whole graph's iteration decision on a shard (after its own pull's
// decide_kernel): the changed mass of all shards, the dense/Wedge rule against
// the whole graph's threshold (execution_bfs.c:132,141), convergence
// (execution_bfs.c:239-251)
__global__ void shard_decide_kernel(DevState s, unsigned long long mass, unsigned long long thr)
{
    Ctrl* c = s.ctrl;
    c->mass = mass;
    c->last_mass = mass;
    c->threshold = thr;
    if (mass == 0ull) {
        c->done = 1u;
        c->loop = 0u;
        c->not_converged = 0u;
    } else if (c->iter >= c->max_iter) {
        c->done = 1u;
        c->loop = 0u;
        c->not_converged = 1u;
    } else {
        c->done = 0u;
        c->loop = 1u;
        c->not_converged = 0u;
        c->mode = mass > thr ? MODE_DENSE : MODE_WEDGE;
    }
}

// the 32-bit copy of SSSP distances a caller imported (dist32_put's rule)
__global__ void narrow_copy_kernel(DevGraph g, DevState s)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    for (uint64_t v = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; v < g.V; v += stride) {
        const unsigned long long d = s.prop64[v];
        s.dist32[v] = d < (unsigned long long)s.narrow_lim ? (uint32_t)d : NONE32;
        if (d >= (unsigned long long)s.narrow_lim && d != NONE64)
            atomicOr(&s.ctrl->narrow_ovf, 1u);
    }
}
}  // namespace wedge

extern "C" {

int wedge_cuda_shard_state(wedge_graph_t* g, int which, void* host, uint64_t bytes, int import)
{
    if (!g || !host || g->built_app < 0 || (which != WEDGE_SHARD_PROPS && which != WEDGE_SHARD_FRONTIER))
        return WEDGE_ERR_ARG;
    const int app = g->built_app;
    if (app == WEDGE_APP_PR)
        return WEDGE_ERR_UNSUPPORTED;
    WEDGE_CHECK(cudaSetDevice(g->device));
    void* dev = nullptr;
    uint64_t need = 0;
    if (which == WEDGE_SHARD_PROPS) {
        dev = app == WEDGE_APP_SSSP ? (void*)g->s.prop64 : (void*)g->s.prop32;
        need = g->g.V * (app == WEDGE_APP_SSSP ? 8ull : 4ull);
    } else {
        Ctrl c;
        int rc = read_ctrl(g, &c);
        if (rc)
            return rc;
        dev = (void*)(c.parity ? g->s.front1 : g->s.front0); /* the bitmap the last pull wrote */
        need = (g->g.V + 31) / 32 * 4ull;
    }
    if (bytes < need)
        return WEDGE_ERR_ARG;
    if (import) {
        WEDGE_CHECK(cudaMemcpyAsync(dev, host, need, cudaMemcpyHostToDevice, g->stream));
        if (which == WEDGE_SHARD_PROPS && g->s.dist32) {
            narrow_copy_kernel<<<grid_for(g->g.V, AUX_THREADS, (uint32_t)g->num_sms * 8u), AUX_THREADS, 0, g->stream>>>(
                g->g, g->s);
            WEDGE_CHECK(cudaGetLastError());
        }
    } else
        WEDGE_CHECK(cudaMemcpyAsync(host, dev, need, cudaMemcpyDeviceToHost, g->stream));
    WEDGE_CHECK(cudaStreamSynchronize(g->stream));
    return WEDGE_OK;
}

int wedge_cuda_shard_decide(wedge_graph_t* g, uint64_t global_mass, uint64_t threshold_pct)
{
    if (!g || g->built_app < 0 || g->built_app == WEDGE_APP_PR || threshold_pct > 100)
        return WEDGE_ERR_ARG;
    WEDGE_CHECK(cudaSetDevice(g->device));
    const unsigned long long thr = (unsigned long long)((g->g.E_thr * threshold_pct) / 100ull);
    shard_decide_kernel<<<1, 1, 0, g->stream>>>(g->s, global_mass, thr);
    WEDGE_CHECK(cudaGetLastError());
    WEDGE_CHECK(cudaStreamSynchronize(g->stream));
    return WEDGE_OK;
}

int wedge_cuda_run_phase(wedge_graph_t* g, int app, int phase, const wedge_params_t* params, uint64_t* active_mass)
{
    int rc = check_params(g, app, params);
    if (rc)
        return rc;
    WEDGE_CHECK(cudaSetDevice(g->device));
    if ((rc = after_exports(g)))
        return rc;
    g->pend_app = -1;
    if ((rc = ensure_state(g, app, params->precision)))
        return rc;
    const DevGraph& dg = g->g;
    g->s.damping = params->damping > 0.0 ? params->damping : 0.875;
    g->s.precision = (uint32_t)params->precision;
    const uint32_t vgrid = aux_grid(g, dg.V);
    Ctrl c;
    switch (phase) {
    case WEDGE_PHASE_INIT:
        if (app == WEDGE_APP_PR && g->s.precision == WEDGE_PREC_FP32C) {
            launch_pr32_init(g, 0u);
        } else if (app == WEDGE_APP_PR) {
            pr_init_kernel<<<vgrid, AUX_THREADS, 0, g->stream>>>(dg, g->s, 0u);
        } else {
            const uint64_t root = params->root < dg.V ? params->root : 0;
            const unsigned long long thr =
                (unsigned long long)((dg.E_thr * (unsigned long long)params->threshold_pct) / 100ull);
            uint64_t cap = params->max_iterations ? params->max_iterations : dg.V + 1;
            launch_init(g, app, root, (uint32_t)params->sched, thr, (uint32_t)(cap > 0x7fffffffull ? 0x7fffffffull : cap));
        }
        break;
    case WEDGE_PHASE_PULL_DENSE:
    case WEDGE_PHASE_PULL_WEDGE: {
        if (app != WEDGE_APP_PR) {
            if ((rc = read_ctrl(g, &c)))
                return rc;
            const uint32_t want = phase == WEDGE_PHASE_PULL_DENSE ? MODE_DENSE : MODE_WEDGE;
            if (c.mode != want && !c.done) {
                if (want == MODE_WEDGE)
                    return WEDGE_ERR_ARG; /* no Wedge frontier was built for this pull */
                WEDGE_CHECK(cudaMemcpyAsync(&g->s.ctrl->mode, &want, sizeof(want), cudaMemcpyHostToDevice, g->stream));
                if (g->s.tile_need) /* its probe lists the tiles whose need bit it sets first */
                    WEDGE_CHECK(cudaMemsetAsync(g->s.tile_need, 0, ((uint64_t)dg.T / 32 + 2) * sizeof(uint32_t), g->stream));
                if (g->s.cand) /* candidates built for a Wedge pull that is not run */
                    WEDGE_CHECK(cudaMemsetAsync(g->s.cand, 0, ((uint64_t)dg.Vne / 32 + 2) * sizeof(uint32_t), g->stream));
            }
        } else if (phase == WEDGE_PHASE_PULL_WEDGE) {
            return WEDGE_ERR_UNSUPPORTED; /* PageRank has no Wedge pull (application.c:154) */
        }
        if (app == WEDGE_APP_PR && g->s.precision == WEDGE_PREC_FP32C) {
            launch_pr32_iteration(g); /* the vertex phase of vertices with in-edges included */
        } else if (app == WEDGE_APP_PR) {
            launch_pull(g, app);
            pr_finish_kernel<<<finish_grid(g, dg), AUX_THREADS, 0, g->stream>>>(
                dg, g->s, g->pull_grid, counters(g));
            launch_pr_total(g);
        } else {
            launch_pull(g, app);
            decide_kernel<<<1, AUX_THREADS, 0, g->stream>>>(dg, g->s, counters(g), pull_slots(g, app), (uint32_t)app);
        }
        break;
    }
    case WEDGE_PHASE_VERTEX_PR:
        if (app != WEDGE_APP_PR)
            return WEDGE_ERR_ARG;
        if (g->s.precision == WEDGE_PREC_FP32C)
            launch_pr32_iso(g); /* the pull finished every other vertex */
        else
            pr_vertex_kernel<<<vgrid, AUX_THREADS, 0, g->stream>>>(dg, g->s);
        break;
    case WEDGE_PHASE_WEDGE_BUILD:
        if (app == WEDGE_APP_PR)
            return WEDGE_ERR_UNSUPPORTED;
        launch_wedge_build(g, dg, app);
        break;
    case WEDGE_PHASE_ADVANCE:
        if (app == WEDGE_APP_PR)
            return WEDGE_ERR_UNSUPPORTED;
        advance_kernel<<<aux_grid(g, (dg.V + 31) / 32), AUX_THREADS, 0, g->stream>>>(dg, g->s, (uint32_t)app);
        break;
    default:
        return WEDGE_ERR_ARG;
    }
    WEDGE_CHECK(cudaGetLastError());
    if ((rc = read_ctrl(g, &c)))
        return rc;
    g->last_app = app;
    if (active_mass)
        *active_mass = app == WEDGE_APP_PR ? 0 : c.mass;
    return WEDGE_OK;
}

int wedge_cuda_read_results(wedge_graph_t* g, void* host_props, uint64_t bytes)
{
    if (!g || !host_props || bytes < 8ull * g->g.V || g->last_app < 0)
        return WEDGE_ERR_ARG;
    WEDGE_CHECK(cudaSetDevice(g->device));
    DevState rs;
    int rc = result_state(g, &rs);
    if (rc)
        return rc;
    // page-locked caller memory is mapped into the device's address space: the
    // export writes the words there directly, with no device copy in between
    cudaPointerAttributes pa;
    if (cudaPointerGetAttributes(&pa, host_props) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer &&
        ((uintptr_t)pa.devicePointer & 7u) == 0u) {
        export_kernel<<<aux_grid(g, g->g.V), AUX_THREADS, 0, g->stream>>>(g->g, rs, (uint32_t)g->last_app,
                                                                         (unsigned long long*)pa.devicePointer);
        WEDGE_CHECK(cudaGetLastError());
        WEDGE_CHECK(cudaStreamSynchronize(g->stream));
        return WEDGE_OK;
    }
    cudaGetLastError(); /* an unregistered pointer is not an error */
    unsigned long long* tmp = nullptr;
    WEDGE_CHECK(cudaMallocAsync((void**)&tmp, 8ull * (g->g.V ? g->g.V : 1), g->stream));
    export_kernel<<<aux_grid(g, g->g.V), AUX_THREADS, 0, g->stream>>>(g->g, rs, (uint32_t)g->last_app, tmp);
    cudaError_t e = cudaMemcpyAsync(host_props, tmp, 8ull * g->g.V, cudaMemcpyDeviceToHost, g->stream);
    cudaFreeAsync(tmp, g->stream);
    WEDGE_CHECK(e);
    WEDGE_CHECK(cudaStreamSynchronize(g->stream));
    return WEDGE_OK;
}

int wedge_cuda_write_output(wedge_graph_t* g, const char* path, int* gpu_formatted, double* format_ms)
{
    if (!g || !path || g->last_app < 0)
        return WEDGE_ERR_ARG;
    WEDGE_CHECK(cudaSetDevice(g->device));
    const uint64_t V = g->g.V;
    const int app = g->last_app;
    const bool on_gpu = app == WEDGE_APP_BFS || app == WEDGE_APP_CC ||
                        (app == WEDGE_APP_SSSP && g->g.weight_kind != WEDGE_WEIGHTS_F64);
    DevState rs;
    int rc = result_state(g, &rs);
    if (rc)
        return rc;
    FILE* f = fopen(path, "w");
    if (!f)
        return WEDGE_ERR_IO;
    float ms = 0.0f;
    if (on_gpu) {
        unsigned long long *len = nullptr, *off = nullptr;
        char* dbuf = nullptr;
        char* hbuf = nullptr;
        unsigned long long total = 0;
        cudaEventRecord(g->ev[0], g->stream);
        if (cudaMalloc((void**)&len, 8ull * (V + 1)) != cudaSuccess || cudaMalloc((void**)&off, 8ull * (V + 1)) != cudaSuccess) {
            rc = WEDGE_ERR_OOM;
        } else {
            cudaMemsetAsync(len + V, 0, 8, g->stream);
            out_len_kernel<<<aux_grid(g, V), AUX_THREADS, 0, g->stream>>>(g->g, rs, (uint32_t)app, len);
            rc = device_scan(g, len, off, V + 1, false);
            if (!rc && (cudaMemcpyAsync(&total, off + V, 8, cudaMemcpyDeviceToHost, g->stream) != cudaSuccess ||
                        cudaStreamSynchronize(g->stream) != cudaSuccess))
                rc = WEDGE_ERR_CUDA;
            if (!rc && (cudaMalloc((void**)&dbuf, total ? total : 1) != cudaSuccess ||
                        cudaMallocHost((void**)&hbuf, total ? total : 1) != cudaSuccess))
                rc = WEDGE_ERR_OOM;
            if (!rc) {
                out_write_kernel<<<aux_grid(g, V), AUX_THREADS, 0, g->stream>>>(g->g, rs, (uint32_t)app, off, dbuf);
                if (cudaMemcpyAsync(hbuf, dbuf, total, cudaMemcpyDeviceToHost, g->stream) != cudaSuccess ||
                    cudaEventRecord(g->ev[1], g->stream) != cudaSuccess || cudaStreamSynchronize(g->stream) != cudaSuccess)
                    rc = WEDGE_ERR_CUDA;
                cudaEventElapsedTime(&ms, g->ev[0], g->ev[1]);
            }
            if (!rc && fwrite(hbuf, 1, total, f) != total)
                rc = WEDGE_ERR_IO;
        }
        cudaFree(len);
        cudaFree(off);
        cudaFree(dbuf);
        if (hbuf)
            cudaFreeHost(hbuf);
    } else {
        /* execution_pr.c:31-35 (%.4le of rank * outdegree'), FP64 SSSP distances (%.17g) */
        uint64_t* props = (uint64_t*)malloc(8 * (V ? V : 1));
        uint64_t* od = (uint64_t*)malloc(8 * (V ? V : 1));
        if (!props || !od) {
            rc = WEDGE_ERR_OOM;
        } else if ((rc = wedge_cuda_read_results(g, props, 8 * V)) == WEDGE_OK &&
                   (rc = wedge_cuda_read_outdegrees(g, od, 8 * V)) == WEDGE_OK) {
            struct timespec t0, t1;
            clock_gettime(CLOCK_MONOTONIC, &t0);
            for (uint64_t v = 0; v < V && !ferror(f); ++v) {
                double d;
                memcpy(&d, &props[v], sizeof(d));
                if (app == WEDGE_APP_PR)
                    fprintf(f, "%llu %.4le\n", (unsigned long long)v, d * (od[v] == 0 ? (double)V : (double)od[v]));
                else
                    fprintf(f, "%llu %.17g\n", (unsigned long long)v, d);
            }
            clock_gettime(CLOCK_MONOTONIC, &t1);
            ms = (float)((t1.tv_sec - t0.tv_sec) * 1e3 + (t1.tv_nsec - t0.tv_nsec) / 1e6);
            if (ferror(f))
                rc = WEDGE_ERR_IO;
        }
        free(props);
        free(od);
    }
    if (fclose(f) != 0 && rc == WEDGE_OK)
        rc = WEDGE_ERR_IO;
    if (gpu_formatted)
        *gpu_formatted = on_gpu ? 1 : 0;
    if (format_ms)
        *format_ms = ms;
    return rc;
}

int wedge_cuda_read_outdegrees(wedge_graph_t* g, uint64_t* host_outdeg, uint64_t bytes)
{
    if (!g || !host_outdeg || bytes < 8ull * g->g.V)
        return WEDGE_ERR_ARG;
    WEDGE_CHECK(cudaSetDevice(g->device));
    unsigned long long* tmp = nullptr;
    WEDGE_CHECK(cudaMallocAsync((void**)&tmp, 8ull * (g->g.V ? g->g.V : 1), g->stream));
    export_outdeg_kernel<<<aux_grid(g, g->g.V), AUX_THREADS, 0, g->stream>>>(g->g, tmp);
    cudaError_t e = cudaMemcpyAsync(host_outdeg, tmp, 8ull * g->g.V, cudaMemcpyDeviceToHost, g->stream);
    cudaFreeAsync(tmp, g->stream);
    WEDGE_CHECK(e);
    WEDGE_CHECK(cudaStreamSynchronize(g->stream));
    return WEDGE_OK;
}

int wedge_cuda_iteration_log(wedge_graph_t* g, wedge_iteration_record_t* out, uint64_t max_records, uint64_t* count)
{
    if (!g || !count || (max_records && !out) || g->last_app < 0 || !g->s.log)
        return WEDGE_ERR_ARG;
    WEDGE_CHECK(cudaSetDevice(g->device));
    Ctrl c;
    int rc = read_ctrl(g, &c);
    if (rc)
        return rc;
    const uint64_t n = c.iter < LOG_CAP ? c.iter : LOG_CAP;
    *count = n;
    const uint64_t m = n < max_records ? n : max_records;
    if (m == 0)
        return WEDGE_OK;
    IterRec* tmp = (IterRec*)malloc(m * sizeof(IterRec));
    if (!tmp)
        return WEDGE_ERR_OOM;
    cudaError_t e = cudaMemcpy(tmp, g->s.log, m * sizeof(IterRec), cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) {
        free(tmp);
        return cuda_status(e);
    }
    for (uint64_t i = 0; i < m; ++i) {
        wedge_iteration_record_t& r = out[i];
        r.active_edges = tmp[i].mass_in;
        r.used_wedge = tmp[i].mode == MODE_WEDGE ? 1u : 0u;
        r.iteration = tmp[i].iter;
        r.pull_ms = g->last_timing ? g->iter_pull_ms[i] : -1.0;
        r.wedge_ms = g->last_timing ? g->iter_wedge_ms[i] : -1.0;
        r.changed_mass = tmp[i].mass_out;
        r.edges_scanned = tmp[i].edges;
        r.tiles_scanned = tmp[i].tiles;
        r.dsts_scanned = tmp[i].dsts;
        r.vertices_activated = tmp[i].activated;
        r.mode = tmp[i].mode;
        r.learned = tmp[i].learned;
        for (int f = 0; f < WEDGE_SCHED_FEATURES; ++f)
            r.features[f] = tmp[i].feat[f];
    }
    free(tmp);
    return WEDGE_OK;
}

int wedge_cuda_set_scheduler(wedge_graph_t* g, const float* blob, uint64_t count)
{
    if (!g || !blob || count != (uint64_t)WEDGE_SCHED_BLOB)
        return WEDGE_ERR_ARG;
    for (uint64_t i = 0; i < (uint64_t)NF; ++i)
        if (!(blob[OFF_SD + i] > 0.0f))
            return WEDGE_ERR_ARG; /* standardisation divides by sd */
    WEDGE_CHECK(cudaSetDevice(g->device));
    if (!g->net) {
        void* p = nullptr;
        WEDGE_CHECK(cudaMalloc(&p, sizeof(float) * WEDGE_SCHED_BLOB));
        g->net = (float*)p;
    }
    WEDGE_CHECK(cudaMemcpyAsync(g->net, blob, sizeof(float) * WEDGE_SCHED_BLOB, cudaMemcpyHostToDevice, g->stream));
    WEDGE_CHECK(cudaStreamSynchronize(g->stream));
    g->s.net = g->net;
    if (g->graph_exec) { /* the captured kernels hold the state by value */
        cudaGraphExecDestroy(g->graph_exec);
        g->graph_exec = nullptr;
        g->graph_app = -1;
    }
    if (g->pr_exec) {
        cudaGraphExecDestroy(g->pr_exec);
        g->pr_exec = nullptr;
    }
    return WEDGE_OK;
}

uint64_t wedge_cuda_num_vertices(const wedge_graph_t* g) { return g ? g->g.V : 0; }
uint64_t wedge_cuda_num_edges(const wedge_graph_t* g) { return g ? g->g.E : 0; }
void* wedge_cuda_stream(const wedge_graph_t* g) { return g ? (void*)g->stream : nullptr; }
void wedge_cuda_free(wedge_graph_t* g) { free_handle(g); }

}  // extern "C"

/* ===================================== allocation-free PageRank iteration */
//
// For callers that cannot allocate device memory -- a host framework that owns
// every device allocation through its own pool, or code running where a
// cudaMalloc would stall or break the caller's stream ordering -- one PageRank
// iteration runs over a CSC the caller already holds in device memory.  The
// caller passes inputs and outputs; the scratch the edge pull needs (the tile
// index, per-tile partial sums of destinations that span tiles, per-block
// totals, the control block) lives in one file-scope static device array of
// fixed size, which every GPU that loads this library holds until exit.
namespace wedge {

constexpr uint64_t NOALLOC_MAX_EDGES = WEDGE_NOALLOC_MAX_EDGES;
constexpr uint32_t NOALLOC_MAX_TILES = (uint32_t)(NOALLOC_MAX_EDGES / TILE);
constexpr uint32_t NOALLOC_MAX_GRID = 2048;
constexpr int NOALLOC_MAX_DEVICES = 64;

struct NoAllocScratch {
    Ctrl ctrl;
    IterRec log[1];
    unsigned int nsplit[2];  // short splits at the front of the split lists, long ones at the back
    unsigned long long block_cnt[NCNT * NOALLOC_MAX_GRID];
    double block_part[NOALLOC_MAX_GRID];
    uint32_t tile_dst0[NOALLOC_MAX_TILES + 1];
    uint32_t dst_start[NOALLOC_MAX_EDGES / 32 + 8];
    uint32_t split_k[NOALLOC_MAX_TILES];
    uint32_t split_t0[NOALLOC_MAX_TILES];
    uint32_t split_t1[NOALLOC_MAX_TILES];
    double head_part[NOALLOC_MAX_TILES];
    double tail_part[NOALLOC_MAX_TILES];
};

// about 6.3 MB on every device that loads the library
static __device__ __align__(256) NoAllocScratch g_noalloc_scratch;

// per-device address of g_noalloc_scratch and the pull grid, set up on the first call
static NoAllocScratch* g_noalloc_ptr[NOALLOC_MAX_DEVICES];
static uint32_t g_noalloc_grid[NOALLOC_MAX_DEVICES];
static pthread_mutex_t g_noalloc_lock = PTHREAD_MUTEX_INITIALIZER;

// control block for one dense pull, tile index (first compressed destination of
// every tile) and a zeroed split count: everything that must start fresh per call
__global__ void noalloc_prepare_kernel(const unsigned long long* dst_off, uint32_t num_dsts, uint32_t T)
{
    NoAllocScratch* sc = &g_noalloc_scratch;
    const uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (tid == 0) {
        Ctrl* c = &sc->ctrl;
        memset(c, 0, sizeof(Ctrl));
        c->mode = MODE_DENSE;
        c->iter = LOG_CAP; /* no per-iteration log in this path */
        sc->nsplit[0] = 0u;
        sc->nsplit[1] = 0u;
    }
    for (uint64_t i = tid; i < (uint64_t)T * TILE / 32 + 1; i += (uint64_t)gridDim.x * blockDim.x)
        sc->dst_start[i] = 0u; /* set by dst_start_kernel next */
    for (uint64_t t = tid; t <= T; t += (uint64_t)gridDim.x * blockDim.x) {
        if (t == T) {
            sc->tile_dst0[t] = num_dsts;
            continue;
        }
        // last destination whose first in-edge is at or before edge t*TILE
        const unsigned long long e = t * (unsigned long long)TILE;
        uint32_t lo = 0, hi = num_dsts; /* dst_off[lo] <= e < dst_off[hi] */
        while (hi - lo > 1) {
            const uint32_t mid = lo + (hi - lo) / 2;
            if (dst_off[mid] <= e)
                lo = mid;
            else
                hi = mid;
        }
        sc->tile_dst0[t] = lo;
    }
}

// total rank and the destinations spanning tiles, as pr_finish_kernel, with the
// split count read from the scratch
__global__ void noalloc_finish_kernel(DevGraph g, DevState s)
{
    NoAllocScratch* sc = &g_noalloc_scratch;
    merge_splits(g, s.acc, sc->split_k, sc->split_t0, sc->split_t1, sc->nsplit[0], sc->nsplit[1], g.T,
                 [&](uint32_t t) { return sc->tail_part[t]; }, [&](uint32_t t) { return sc->head_part[t]; });
}

static int noalloc_setup(int dev, NoAllocScratch** sc, uint32_t* grid)
{
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return WEDGE_ERR_UNSUPPORTED;
    pthread_mutex_lock(&g_noalloc_lock);
    int rc = WEDGE_OK;
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch); /* device `dev` is current */
        int sms = 0, blocks = 0;
        if (e == cudaSuccess)
            e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (e == cudaSuccess)
            e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, pull_kernel<WEDGE_APP_PR, PullEpl<WEDGE_APP_PR>::value>, PULL_THREADS, 0);
        if (e != cudaSuccess) {
            rc = cuda_status(e);
        } else {
            uint32_t grid = (uint32_t)(sms * (blocks > 0 ? blocks : 1));
            g_noalloc_grid[dev] = grid < NOALLOC_MAX_GRID ? grid : NOALLOC_MAX_GRID;
            g_noalloc_ptr[dev] = (NoAllocScratch*)p;
        }
    }
    *sc = g_noalloc_ptr[dev];
    *grid = g_noalloc_grid[dev];
    pthread_mutex_unlock(&g_noalloc_lock);
    return rc;
}

}  // namespace wedge

extern "C" int wedge_cuda_pr_iteration_noalloc(uint64_t num_vertices, uint64_t num_dsts, uint64_t num_edges,
                                               const uint64_t* dst_off, const uint32_t* dst_id, const uint32_t* src,
                                               const uint32_t* outdeg, const double* rank_in, double* rank_out,
                                               double damping, void* stream)
{
    using namespace wedge;
    if (num_edges > NOALLOC_MAX_EDGES || num_dsts > num_edges || num_vertices == 0 || num_vertices > 0xFFFFFFFEull ||
        num_dsts > num_vertices)
        return WEDGE_ERR_ARG; /* beyond the static scratch, or inconsistent sizes */
    if (!dst_off || !dst_id || !src || !outdeg || !rank_in || !rank_out || ((uintptr_t)src & 15u) ||
        (num_edges && !num_dsts))
        return WEDGE_ERR_ARG;
    int dev = 0;
    WEDGE_CHECK(cudaGetDevice(&dev));
    NoAllocScratch* sc = nullptr;
    uint32_t grid = 0;
    int rc = noalloc_setup(dev, &sc, &grid);
    if (rc)
        return rc;
    cudaStream_t st = (cudaStream_t)stream;
    const uint32_t T = (uint32_t)((num_edges + TILE - 1) / TILE);
    DevGraph g;
    memset(&g, 0, sizeof(g));
    g.V = num_vertices;
    g.E = num_edges;
    g.Epad = (uint64_t)T * TILE;
    g.Vne = (uint32_t)num_dsts;
    g.T = T;
    g.weight_kind = WEDGE_WEIGHTS_NONE;
    g.src = src;
    g.dst_id = dst_id;
    g.dst_off = (const unsigned long long*)dst_off;
    g.tile_dst0 = sc->tile_dst0;
    g.dst_start = sc->dst_start;
    g.outdeg = outdeg;
    g.split_k = sc->split_k;
    g.split_t0 = sc->split_t0;
    g.split_t1 = sc->split_t1;
    DevState s;
    memset(&s, 0, sizeof(s));
    s.ctrl = &sc->ctrl;
    s.log = sc->log;
    s.head_part = sc->head_part;
    s.tail_part = sc->tail_part;
    s.block_part = sc->block_part;
    s.damping = damping > 0.0 ? damping : 0.875;
    s.precision = WEDGE_PREC_FP64;
    s.app = WEDGE_APP_PR;
    s.acc = rank_out; /* accumulators first, ranks after the vertex phase */
    const uint32_t aux = (uint32_t)grid_for(num_vertices > T ? num_vertices : (uint64_t)T + 1, AUX_THREADS, grid * 2u);
    noalloc_prepare_kernel<<<aux, AUX_THREADS, 0, st>>>(g.dst_off, g.Vne, T);
    if (num_dsts)
        dst_start_kernel<<<grid_for(num_dsts, AUX_THREADS, grid * 2u), AUX_THREADS, 0, st>>>(g.dst_off, g.Vne,
                                                                                          sc->dst_start);
    if (num_dsts)
        split_kernel<<<grid_for(num_dsts, AUX_THREADS, grid * 2u), AUX_THREADS, 0, st>>>(
            g.dst_off, g.Vne, T, TILE, sc->split_k, sc->split_t0, sc->split_t1, sc->nsplit);
    WEDGE_CHECK(cudaMemsetAsync(rank_out, 0, num_vertices * sizeof(double), st));
    DevState sp = s;
    sp.rank = (double*)rank_in; /* gathered by the pull */
    if (T)
        pull_kernel<WEDGE_APP_PR, PullEpl<WEDGE_APP_PR>::value><<<grid, PULL_THREADS, 0, st>>>(g, sp, sc->block_cnt,
                                                                                           PHASE_ALL); /* no hub cache */
    noalloc_finish_kernel<<<grid_for((uint64_t)T + 1, AUX_THREADS, grid * 2u), AUX_THREADS, 0, st>>>(g, s);
    pr_total_kernel<<<grid_for(num_vertices, AUX_THREADS, NOALLOC_MAX_GRID < grid * 2u ? NOALLOC_MAX_GRID : grid * 2u),
                      AUX_THREADS, 0, st>>>(s.acc, num_vertices, sc->block_part, &sc->ctrl);
    DevState sv = s;
    sv.rank = rank_out;
    pr_vertex_kernel<<<grid_for(num_vertices, AUX_THREADS, grid * 2u), AUX_THREADS, 0, st>>>(g, sv);
    WEDGE_CHECK(cudaGetLastError());
    return WEDGE_OK;
}
