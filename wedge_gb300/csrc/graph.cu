// Graph ingest for the sm_103a engine: the Wedge binary edge-list file (from
// disk or from a host image), host edge arrays, the reference's in-memory
// edge-vector list, and the synthetic generators.  Every path ends in
// build_from_device_edges (engine.cu), which lays out the device CSC.
//
// Reference correspondence: graph_data_read_from_file (graphdata.c:946-1133)
// reads the file twice through a 3 MiB double buffer; here the records stream
// once through two pinned staging buffers, each chunk copied to the device and
// unpacked by a kernel while the next chunk is read.
#include <cub/device/device_radix_sort.cuh>
#include <cub/device/device_scan.cuh>

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "engine.cuh"

namespace wedge {

constexpr uint64_t STAGE_RECORDS = 1ull << 22; /* records per staging chunk */
constexpr uint64_t MAX_VERTICES = 0xFFFFFFFEull;

static uint32_t grid_cap(int sms) { return (uint32_t)sms * 16u; }

static uint32_t grid_of(uint64_t n, int sms)
{
    uint64_t b = (n + 255) / 256;
    if (b < 1)
        b = 1;
    const uint64_t cap = grid_cap(sms);
    return (uint32_t)(b < cap ? b : cap);
}

// unpack `n` records of `tup` words starting at record `first`
__global__ void unpack_records_kernel(const unsigned long long* rec, uint64_t n, uint32_t tup, uint64_t first,
                                      uint64_t V, uint32_t* src, uint32_t* dst, unsigned long long* w, int* err)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long s = rec[i * tup], d = rec[i * tup + 1];
        if (s >= V || d >= V) {
            atomicOr(err, 1);
            continue;
        }
        src[first + i] = (uint32_t)s;
        dst[first + i] = (uint32_t)d;
        if (w)
            w[first + i] = rec[i * tup + 2];
    }
}

struct RecordReader {
    FILE* f;
    const unsigned char* image;
    uint64_t pos;
};

static int fetch(RecordReader& r, void* dst, uint64_t bytes)
{
    if (r.f)
        return fread(dst, 1, bytes, r.f) == bytes ? WEDGE_OK : WEDGE_ERR_IO;
    memcpy(dst, r.image + r.pos, bytes);
    r.pos += bytes;
    return WEDGE_OK;
}

static int alloc_edges(uint64_t E, bool weighted, uint32_t** src, uint32_t** dst, unsigned long long** w)
{
    const uint64_t Epad = (E + MAX_TILE_E - 1) / MAX_TILE_E * MAX_TILE_E;
    *src = nullptr;
    *dst = nullptr;
    *w = nullptr;
    WEDGE_CHECK(cudaMalloc((void**)src, (Epad ? Epad : MAX_TILE_E) * sizeof(uint32_t)));
    WEDGE_CHECK(cudaMalloc((void**)dst, (E ? E : 1) * sizeof(uint32_t)));
    if (weighted)
        WEDGE_CHECK(cudaMalloc((void**)w, (Epad ? Epad : MAX_TILE_E) * sizeof(unsigned long long)));
    return WEDGE_OK;
}

// streams E records through two pinned staging buffers into device edge arrays
static int ingest_records(wedge_graph* h, RecordReader& rd, uint64_t V, uint64_t E, uint32_t tup, int weight_kind)
{
    uint32_t *d_src, *d_dst;
    unsigned long long* d_w;
    int rc = alloc_edges(E, tup == 3, &d_src, &d_dst, &d_w);
    if (rc)
        return rc;
    if ((rc = track(h, d_src)))
        return rc;
    if (d_w && (rc = track(h, d_w)))
        return rc;
    const uint64_t chunk = E < STAGE_RECORDS ? (E ? E : 1) : STAGE_RECORDS;
    const size_t chunk_bytes = chunk * tup * sizeof(unsigned long long);
    unsigned long long *pin[2] = {nullptr, nullptr}, *dev[2] = {nullptr, nullptr};
    cudaEvent_t done[2];
    int* d_err = nullptr;
    WEDGE_CHECK(cudaMallocHost((void**)&pin[0], chunk_bytes));
    WEDGE_CHECK(cudaMallocHost((void**)&pin[1], chunk_bytes));
    WEDGE_CHECK(cudaMalloc((void**)&dev[0], chunk_bytes));
    WEDGE_CHECK(cudaMalloc((void**)&dev[1], chunk_bytes));
    WEDGE_CHECK(cudaMalloc((void**)&d_err, sizeof(int)));
    WEDGE_CHECK(cudaMemsetAsync(d_err, 0, sizeof(int), h->stream));
    WEDGE_CHECK(cudaEventCreateWithFlags(&done[0], cudaEventDisableTiming));
    WEDGE_CHECK(cudaEventCreateWithFlags(&done[1], cudaEventDisableTiming));
    int b = 0;
    for (uint64_t first = 0; first < E && rc == WEDGE_OK; first += chunk, b ^= 1) {
        const uint64_t n = (E - first) < chunk ? (E - first) : chunk;
        cudaEventSynchronize(done[b]); /* staging buffer b is free again */
        if ((rc = fetch(rd, pin[b], n * tup * sizeof(unsigned long long))))
            break;
        cudaMemcpyAsync(dev[b], pin[b], n * tup * sizeof(unsigned long long), cudaMemcpyHostToDevice, h->stream);
        unpack_records_kernel<<<grid_of(n, h->num_sms), 256, 0, h->stream>>>(dev[b], n, tup, first, V, d_src, d_dst,
                                                                              d_w, d_err);
        cudaEventRecord(done[b], h->stream);
    }
    int herr = 0;
    cudaMemcpyAsync(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost, h->stream);
    cudaError_t ce = cudaStreamSynchronize(h->stream);
    cudaFreeHost(pin[0]);
    cudaFreeHost(pin[1]);
    cudaFree(dev[0]);
    cudaFree(dev[1]);
    cudaFree(d_err);
    cudaEventDestroy(done[0]);
    cudaEventDestroy(done[1]);
    if (rc) {
        cudaFree(d_dst);
        return rc;
    }
    if (ce != cudaSuccess) {
        cudaFree(d_dst);
        return cuda_status(ce);
    }
    if (herr) {
        cudaFree(d_dst);
        return WEDGE_ERR_FORMAT;
    }
    return build_from_device_edges(h, V, E, d_src, d_dst, d_w, tup == 3 ? weight_kind : WEDGE_WEIGHTS_NONE);
}

static int normalise_weights(int app, int weight_kind, uint32_t* tup, int* kind)
{
    if (app < WEDGE_APP_BFS || app > WEDGE_APP_SSSP)
        return WEDGE_ERR_ARG;
    if (app == WEDGE_APP_SSSP) { /* application.c:171: SSSP reads (src, dst, weight) */
        *tup = 3;
        *kind = (weight_kind == WEDGE_WEIGHTS_F64) ? WEDGE_WEIGHTS_F64 : WEDGE_WEIGHTS_U64;
    } else {
        *tup = 2;
        *kind = WEDGE_WEIGHTS_NONE;
    }
    return WEDGE_OK;
}

/* ---------------------------------------------------------------- generators */

__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

__device__ __forceinline__ unsigned long long draw(unsigned long long seed, unsigned long long item, unsigned int word)
{
    return mix64(mix64(seed) + ((item << 4) | (word & 15u)));
}

// R-MAT: one quadrant per bit level, most significant first (same rule as the
// CPU generator); key = dst << sbits | src, plus the reverse pair when symmetrising
__global__ void rmat_kernel(uint32_t scale, unsigned long long ta, unsigned long long tab, unsigned long long tabc,
                            unsigned long long seed, uint64_t E0, int sym, uint32_t sbits, unsigned long long* keys)
{
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E0; e += (uint64_t)gridDim.x * blockDim.x) {
        uint32_t s = 0, d = 0;
        unsigned long long hv = 0;
        for (uint32_t l = 0; l < scale; ++l) {
            if ((l & 1u) == 0)
                hv = draw(seed, e, l >> 1);
            const unsigned long long u = (l & 1u) ? (hv >> 32) : (hv & 0xffffffffull);
            const uint32_t bit = 1u << (scale - 1 - l);
            if (u < ta) {
            } else if (u < tab) {
                d |= bit;
            } else if (u < tabc) {
                s |= bit;
            } else {
                s |= bit;
                d |= bit;
            }
        }
        keys[e] = ((unsigned long long)d << sbits) | s;
        if (sym)
            keys[E0 + e] = ((unsigned long long)s << sbits) | d;
    }
}

// 4-neighbour grid (both directions) + long-range pairs, same multiset as the CPU generator
__global__ void grid_kernel(uint64_t side, uint64_t lr, unsigned long long seed, uint32_t sbits, unsigned long long* keys)
{
    const uint64_t H = 2ull * side * (side - 1ull);
    const uint64_t base = 2ull * H;
    const uint64_t V = side * side;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < base + lr;
         i += (uint64_t)gridDim.x * blockDim.x) {
        uint64_t s, d;
        if (i < H) {
            const uint64_t p = i >> 1, r = p / (side - 1), c = p % (side - 1), v = r * side + c;
            s = (i & 1) ? v + 1 : v;
            d = (i & 1) ? v : v + 1;
        } else if (i < base) {
            const uint64_t p = (i - H) >> 1, r = p / side, c = p % side, v = r * side + c;
            s = ((i - H) & 1) ? v + side : v;
            d = ((i - H) & 1) ? v : v + side;
        } else {
            const uint64_t j = i - base;
            s = __umul64hi(draw(seed, j, 0), V);
            d = __umul64hi(draw(seed, j, 1), V);
        }
        keys[i] = (d << sbits) | s;
    }
}

__device__ __forceinline__ unsigned long long weight_word(uint32_t s, uint32_t d, int kind)
{
    const unsigned long long h = (((unsigned long long)s << 32) | d) * 0x9E3779B97F4A7C15ull;
    if (kind == WEDGE_WEIGHTS_F64)
        return (unsigned long long)__double_as_longlong(__dmul_rn(__ull2double_rn(h), 0x1p-64));
    return 1ull + (((h >> 32) * 255ull) >> 32);
}

__global__ void unpack_keys_kernel(const unsigned long long* keys, uint64_t E, uint32_t sbits, int kind, uint32_t* src,
                                   uint32_t* dst, unsigned long long* w)
{
    const unsigned long long mask = (1ull << sbits) - 1ull;
    for (uint64_t e = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; e < E; e += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long k = keys[e];
        const uint32_t s = (uint32_t)(k & mask), d = (uint32_t)(k >> sbits);
        src[e] = s;
        dst[e] = d;
        if (w)
            w[e] = weight_word(s, d, kind);
    }
}

static uint32_t bits_for(uint64_t V)
{
    uint32_t b = 1;
    while (b < 63 && (1ull << b) < V)
        ++b;
    return b;
}

// sorts the (dst, src) keys, unpacks them into edge arrays and builds the CSC
static int build_from_keys(wedge_graph* h, uint64_t V, uint64_t E, unsigned long long* keys, uint32_t sbits,
                           int weight_kind)
{
    cudaStream_t st = h->stream;
    unsigned long long* alt = nullptr;
    WEDGE_CHECK(cudaMalloc((void**)&alt, (E ? E : 1) * sizeof(unsigned long long)));
    cub::DoubleBuffer<unsigned long long> db(keys, alt);
    size_t tb = 0;
    WEDGE_CHECK(cub::DeviceRadixSort::SortKeys(nullptr, tb, db, (long long)E, 0, (int)(2 * sbits), st));
    void* tmp = nullptr;
    WEDGE_CHECK(cudaMalloc(&tmp, tb ? tb : 1));
    WEDGE_CHECK(cub::DeviceRadixSort::SortKeys(tmp, tb, db, (long long)E, 0, (int)(2 * sbits), st));
    uint32_t *d_src, *d_dst;
    unsigned long long* d_w;
    int rc = alloc_edges(E, weight_kind != WEDGE_WEIGHTS_NONE, &d_src, &d_dst, &d_w);
    if (rc)
        return rc;
    if ((rc = track(h, d_src)) || (d_w && (rc = track(h, d_w))))
        return rc;
    if (E)
        unpack_keys_kernel<<<grid_of(E, h->num_sms), 256, 0, st>>>(db.Current(), E, sbits, weight_kind, d_src, d_dst,
                                                                     d_w);
    WEDGE_CHECK(cudaStreamSynchronize(st));
    cudaFree(tmp);
    cudaFree(alt);
    cudaFree(keys);
    WEDGE_CHECK(cudaGetLastError());
    return build_from_device_edges(h, V, E, d_src, d_dst, d_w, weight_kind);
}

}  // namespace wedge

using namespace wedge;

extern "C" {

int wedge_cuda_load_graph_ex(const char* path, int app, int weight_kind, wedge_graph_t** out)
{
    if (!path || !out)
        return WEDGE_ERR_ARG;
    *out = nullptr;
    uint32_t tup;
    int kind;
    int rc = normalise_weights(app, weight_kind, &tup, &kind);
    if (rc)
        return rc;
    FILE* f = fopen(path, "rb");
    if (!f)
        return WEDGE_ERR_IO;
    unsigned long long hdr[2];
    if (fread(hdr, 8, 2, f) != 2) {
        fclose(f);
        return WEDGE_ERR_FORMAT;
    }
    fseek(f, 0, SEEK_END);
    const long long fsize = ftell(f);
    fseek(f, 16, SEEK_SET);
    const uint64_t V = hdr[0], E = hdr[1];
    /* exact size check, graphdata.c:962-979 */
    if (E > (1ull << 40) || fsize < 0 || (uint64_t)fsize != 16ull + E * tup * 8ull || V == 0 || V > MAX_VERTICES) {
        fclose(f);
        return WEDGE_ERR_FORMAT;
    }
    wedge_graph* h = nullptr;
    if ((rc = new_handle(&h))) {
        fclose(f);
        return rc;
    }
    RecordReader rd{f, nullptr, 0};
    rc = ingest_records(h, rd, V, E, tup, kind);
    fclose(f);
    if (rc) {
        free_handle(h);
        return rc;
    }
    *out = h;
    return WEDGE_OK;
}

int wedge_cuda_load_graph(const char* path, int app, wedge_graph_t** out)
{
    return wedge_cuda_load_graph_ex(path, app, WEDGE_WEIGHTS_U64, out);
}

int wedge_cuda_load_graph_image(const void* image, uint64_t bytes, int app, int weight_kind, wedge_graph_t** out)
{
    if (!image || !out)
        return WEDGE_ERR_ARG;
    *out = nullptr;
    uint32_t tup;
    int kind;
    int rc = normalise_weights(app, weight_kind, &tup, &kind);
    if (rc)
        return rc;
    if (bytes < 16)
        return WEDGE_ERR_FORMAT;
    unsigned long long hdr[2];
    memcpy(hdr, image, 16);
    const uint64_t V = hdr[0], E = hdr[1];
    if (E > (1ull << 40) || bytes != 16ull + E * tup * 8ull || V == 0 || V > MAX_VERTICES)
        return WEDGE_ERR_FORMAT;
    wedge_graph* h = nullptr;
    if ((rc = new_handle(&h)))
        return rc;
    RecordReader rd{nullptr, (const unsigned char*)image, 16};
    rc = ingest_records(h, rd, V, E, tup, kind);
    if (rc) {
        free_handle(h);
        return rc;
    }
    *out = h;
    return WEDGE_OK;
}

int wedge_cuda_load_shard(uint64_t num_vertices, uint64_t num_edges, const uint32_t* src, const uint32_t* dst,
                          const uint64_t* weights, int weight_kind, const uint64_t* global_outdeg,
                          uint64_t global_edges, wedge_graph_t** out)
{
    if (!out || (num_edges && (!src || !dst)) || !global_outdeg || num_vertices == 0 || num_vertices > MAX_VERTICES ||
        global_edges < num_edges)
        return WEDGE_ERR_ARG;
    if (weights && weight_kind == WEDGE_WEIGHTS_NONE)
        return WEDGE_ERR_ARG;
    *out = nullptr;
    uint32_t* deg32 = (uint32_t*)malloc(num_vertices * sizeof(uint32_t));
    if (!deg32)
        return WEDGE_ERR_OOM;
    for (uint64_t v = 0; v < num_vertices; ++v) {
        if (global_outdeg[v] > 0xFFFFFFFFull) {
            free(deg32);
            return WEDGE_ERR_FORMAT;
        }
        deg32[v] = (uint32_t)global_outdeg[v];
    }
    wedge_graph* h = nullptr;
    int rc = new_handle(&h);
    if (rc) {
        free(deg32);
        return rc;
    }
    uint32_t *d_src, *d_dst, *d_deg = nullptr;
    unsigned long long* d_w;
    const uint64_t E = num_edges;
    if ((rc = alloc_edges(E, weights != nullptr, &d_src, &d_dst, &d_w)) || (rc = track(h, d_src)) ||
        (d_w && (rc = track(h, d_w)))) {
        free(deg32);
        free_handle(h);
        return rc;
    }
    cudaError_t e0 = cudaMalloc((void**)&d_deg, num_vertices * sizeof(uint32_t));
    cudaError_t e1 = cudaMemcpyAsync(d_src, src, E * 4, cudaMemcpyHostToDevice, h->stream);
    cudaError_t e2 = cudaMemcpyAsync(d_dst, dst, E * 4, cudaMemcpyHostToDevice, h->stream);
    cudaError_t e3 = weights ? cudaMemcpyAsync(d_w, weights, E * 8, cudaMemcpyHostToDevice, h->stream) : cudaSuccess;
    cudaError_t e4 = e0 == cudaSuccess ? cudaMemcpyAsync(d_deg, deg32, num_vertices * 4, cudaMemcpyHostToDevice, h->stream)
                                       : e0;
    cudaError_t e5 = cudaStreamSynchronize(h->stream);
    free(deg32);
    if (e0 != cudaSuccess || e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess || e4 != cudaSuccess ||
        e5 != cudaSuccess) {
        cudaFree(d_deg);
        cudaFree(d_dst);
        free_handle(h);
        return e0 == cudaErrorMemoryAllocation ? WEDGE_ERR_OOM : WEDGE_ERR_CUDA;
    }
    rc = build_from_device_edges(h, num_vertices, E, d_src, d_dst, d_w, weights ? weight_kind : WEDGE_WEIGHTS_NONE, d_deg);
    cudaStreamSynchronize(h->stream);
    cudaFree(d_deg);
    if (rc) {
        free_handle(h);
        return rc;
    }
    h->g.E_thr = global_edges;
    h->g.shard = 1u;
    *out = h;
    return WEDGE_OK;
}

int wedge_cuda_load_edges(uint64_t num_vertices, uint64_t num_edges, const uint32_t* src, const uint32_t* dst,
                          const uint64_t* weights, int weight_kind, wedge_graph_t** out)
{
    if (!out || (num_edges && (!src || !dst)) || num_vertices == 0 || num_vertices > MAX_VERTICES)
        return WEDGE_ERR_ARG;
    if (weights && weight_kind == WEDGE_WEIGHTS_NONE)
        return WEDGE_ERR_ARG;
    *out = nullptr;
    wedge_graph* h = nullptr;
    int rc = new_handle(&h);
    if (rc)
        return rc;
    uint32_t *d_src, *d_dst;
    unsigned long long* d_w;
    const uint64_t E = num_edges;
    if ((rc = alloc_edges(E, weights != nullptr, &d_src, &d_dst, &d_w)) || (rc = track(h, d_src)) ||
        (d_w && (rc = track(h, d_w)))) {
        free_handle(h);
        return rc;
    }
    cudaError_t e1 = cudaMemcpyAsync(d_src, src, E * 4, cudaMemcpyHostToDevice, h->stream);
    cudaError_t e2 = cudaMemcpyAsync(d_dst, dst, E * 4, cudaMemcpyHostToDevice, h->stream);
    cudaError_t e3 = weights ? cudaMemcpyAsync(d_w, weights, E * 8, cudaMemcpyHostToDevice, h->stream) : cudaSuccess;
    if (e1 != cudaSuccess || e2 != cudaSuccess || e3 != cudaSuccess) {
        cudaFree(d_dst);
        free_handle(h);
        return WEDGE_ERR_CUDA;
    }
    rc = build_from_device_edges(h, num_vertices, E, d_src, d_dst, d_w, weights ? weight_kind : WEDGE_WEIGHTS_NONE);
    if (rc) {
        free_handle(h);
        return rc;
    }
    *out = h;
    return WEDGE_OK;
}

}  // extern "C"

namespace wedge {

// number of valid lanes of each edge vector (graphdata.c:212-243 layout)
__global__ void vec_count_kernel(const unsigned long long* vecs, uint64_t nvec, uint32_t words, uint32_t* cnt)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nvec; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long* v = vecs + i * words;
        cnt[i] = (uint32_t)((v[0] >> 63) + (v[1] >> 63) + (v[2] >> 63) + (v[3] >> 63));
    }
}

// extract_destination_vertex (phase_edge_pull_bfs.c:23) and the 48-bit sources
__global__ void vec_decode_kernel(const unsigned long long* vecs, uint64_t nvec, uint32_t words, const uint64_t* pos,
                                  uint64_t V, uint32_t* src, uint32_t* dst, unsigned long long* w, int* err)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < nvec; i += (uint64_t)gridDim.x * blockDim.x) {
        const unsigned long long* v = vecs + i * words;
        const unsigned long long d = ((v[0] >> 48) & 0x7fffull) | (((v[1] >> 48) & 0x7fffull) << 15) |
                                     (((v[2] >> 48) & 0x7fffull) << 30) | (((v[3] >> 48) & 0x7ull) << 45);
        uint64_t o = pos[i];
        for (int k = 0; k < 4; ++k) {
            if (!(v[k] >> 63))
                continue;
            const unsigned long long s = v[k] & 0x0000ffffffffffffull;
            if (s >= V || d >= V) {
                atomicOr(err, 1);
            } else {
                src[o] = (uint32_t)s;
                dst[o] = (uint32_t)d;
                if (w)
                    w[o] = v[4 + k];
            }
            ++o;
        }
    }
}

}  // namespace wedge

extern "C" {

int wedge_cuda_load_edge_vectors(uint64_t num_vertices, const uint64_t* vectors, uint64_t num_vectors, int weighted,
                                 int weight_kind, wedge_graph_t** out)
{
    if (!out || (num_vectors && !vectors) || num_vertices == 0 || num_vertices > MAX_VERTICES)
        return WEDGE_ERR_ARG;
    *out = nullptr;
    if (weighted && weight_kind == WEDGE_WEIGHTS_NONE)
        weight_kind = WEDGE_WEIGHTS_U64;
    wedge_graph* h = nullptr;
    int rc = new_handle(&h);
    if (rc)
        return rc;
    cudaStream_t st = h->stream;
    const uint32_t words = weighted ? 8 : 4;
    unsigned long long* d_vec = nullptr;
    uint32_t* d_cnt = nullptr;
    uint64_t* d_pos = nullptr;
    int* d_err = nullptr;
    const uint64_t nv = num_vectors ? num_vectors : 1;
    if (cudaMalloc((void**)&d_vec, nv * words * 8) != cudaSuccess || cudaMalloc((void**)&d_cnt, nv * 4) != cudaSuccess ||
        cudaMalloc((void**)&d_pos, (nv + 1) * 8) != cudaSuccess || cudaMalloc((void**)&d_err, 4) != cudaSuccess) {
        cudaFree(d_vec);
        cudaFree(d_cnt);
        cudaFree(d_pos);
        free_handle(h);
        return WEDGE_ERR_OOM;
    }
    cudaMemsetAsync(d_err, 0, 4, st);
    cudaMemsetAsync(d_pos, 0, 8, st);
    if (num_vectors) {
        cudaMemcpyAsync(d_vec, vectors, num_vectors * words * 8, cudaMemcpyHostToDevice, st);
        vec_count_kernel<<<grid_of(num_vectors, h->num_sms), 256, 0, st>>>(d_vec, num_vectors, words, d_cnt);
        size_t tb = 0;
        cub::DeviceScan::ExclusiveSum(nullptr, tb, d_cnt, d_pos, (long long)num_vectors, st);
        void* tmp = nullptr;
        cudaMalloc(&tmp, tb ? tb : 1);
        /* first edge of each vector; the total is the last position plus the last count */
        cub::DeviceScan::ExclusiveSum(tmp, tb, d_cnt, d_pos, (long long)num_vectors, st);
        cudaStreamSynchronize(st);
        cudaFree(tmp);
    }
    uint64_t E = 0;
    if (num_vectors) {
        uint64_t last_pos = 0;
        uint32_t last_cnt = 0;
        cudaMemcpy(&last_pos, d_pos + (num_vectors - 1), 8, cudaMemcpyDeviceToHost);
        cudaMemcpy(&last_cnt, d_cnt + (num_vectors - 1), 4, cudaMemcpyDeviceToHost);
        E = last_pos + last_cnt;
    }
    uint32_t *d_src, *d_dst;
    unsigned long long* d_w;
    if ((rc = alloc_edges(E, weighted != 0, &d_src, &d_dst, &d_w)) || (rc = track(h, d_src)) ||
        (d_w && (rc = track(h, d_w)))) {
        cudaFree(d_vec);
        cudaFree(d_cnt);
        cudaFree(d_pos);
        cudaFree(d_err);
        free_handle(h);
        return rc;
    }
    if (num_vectors)
        vec_decode_kernel<<<grid_of(num_vectors, h->num_sms), 256, 0, st>>>(d_vec, num_vectors, words, d_pos,
                                                                            num_vertices, d_src, d_dst, d_w, d_err);
    int herr = 0;
    cudaMemcpyAsync(&herr, d_err, 4, cudaMemcpyDeviceToHost, st);
    cudaError_t ce = cudaStreamSynchronize(st);
    cudaFree(d_vec);
    cudaFree(d_cnt);
    cudaFree(d_pos);
    cudaFree(d_err);
    if (ce != cudaSuccess || herr) {
        cudaFree(d_dst);
        free_handle(h);
        return ce != cudaSuccess ? WEDGE_ERR_CUDA : WEDGE_ERR_FORMAT;
    }
    rc = build_from_device_edges(h, num_vertices, E, d_src, d_dst, d_w, weighted ? weight_kind : WEDGE_WEIGHTS_NONE);
    if (rc) {
        free_handle(h);
        return rc;
    }
    *out = h;
    return WEDGE_OK;
}

int wedge_cuda_generate_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                             int symmetrise, int weight_kind, wedge_graph_t** out)
{
    if (!out || scale < 1 || scale > 31 || edge_factor == 0 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
        return WEDGE_ERR_ARG;
    *out = nullptr;
    const uint64_t V = 1ull << scale;
    const uint64_t E0 = (uint64_t)edge_factor << scale;
    const uint64_t E = symmetrise ? 2 * E0 : E0;
    wedge_graph* h = nullptr;
    int rc = new_handle(&h);
    if (rc)
        return rc;
    unsigned long long* keys = nullptr;
    if (cudaMalloc((void**)&keys, E * sizeof(unsigned long long)) != cudaSuccess) {
        free_handle(h);
        return WEDGE_ERR_OOM;
    }
    /* thresholds exactly as the CPU generator computes them */
    const unsigned long long ta = (unsigned long long)(a * 4294967296.0);
    const unsigned long long tab = (unsigned long long)((a + b) * 4294967296.0);
    const unsigned long long tabc = (unsigned long long)((a + b + c) * 4294967296.0);
    rmat_kernel<<<grid_of(E0, h->num_sms), 256, 0, h->stream>>>(scale, ta, tab, tabc, seed, E0, symmetrise ? 1 : 0, scale,
                                                                keys);
    rc = build_from_keys(h, V, E, keys, scale, weight_kind);
    if (rc) {
        free_handle(h);
        return rc;
    }
    *out = h;
    return WEDGE_OK;
}

int wedge_cuda_generate_grid(uint32_t side, double long_range_frac, uint64_t seed, int weight_kind, wedge_graph_t** out)
{
    if (!out || side < 2 || side > 65535 || long_range_frac < 0.0)
        return WEDGE_ERR_ARG;
    *out = nullptr;
    const uint64_t V = (uint64_t)side * side;
    const uint64_t base = 4ull * side * (side - 1ull);
    const uint64_t lr = (uint64_t)(long_range_frac * (double)base);
    const uint64_t E = base + lr;
    const uint32_t sbits = bits_for(V);
    wedge_graph* h = nullptr;
    int rc = new_handle(&h);
    if (rc)
        return rc;
    unsigned long long* keys = nullptr;
    if (cudaMalloc((void**)&keys, E * sizeof(unsigned long long)) != cudaSuccess) {
        free_handle(h);
        return WEDGE_ERR_OOM;
    }
    grid_kernel<<<grid_of(E, h->num_sms), 256, 0, h->stream>>>(side, lr, seed, sbits, keys);
    rc = build_from_keys(h, V, E, keys, sbits, weight_kind);
    if (rc) {
        free_handle(h);
        return rc;
    }
    *out = h;
    return WEDGE_OK;
}

// generated keys -> (dst, src)-sorted host arrays
static int keys_to_host(unsigned long long* keys, uint64_t E, uint32_t sbits, uint32_t* src, uint32_t* dst)
{
    cudaStream_t st = nullptr;
    unsigned long long* alt = nullptr;
    uint32_t *ds = nullptr, *dd = nullptr;
    void* tmp = nullptr;
    int rc = WEDGE_OK;
    cub::DoubleBuffer<unsigned long long> db(keys, nullptr);
    size_t tb = 0;
    if (cudaMalloc((void**)&alt, (E ? E : 1) * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc((void**)&ds, (E ? E : 1) * sizeof(uint32_t)) != cudaSuccess ||
        cudaMalloc((void**)&dd, (E ? E : 1) * sizeof(uint32_t)) != cudaSuccess) {
        rc = WEDGE_ERR_OOM;
    } else {
        db = cub::DoubleBuffer<unsigned long long>(keys, alt);
        if (cub::DeviceRadixSort::SortKeys(nullptr, tb, db, (long long)E, 0, (int)(2 * sbits), st) != cudaSuccess ||
            cudaMalloc(&tmp, tb ? tb : 1) != cudaSuccess ||
            cub::DeviceRadixSort::SortKeys(tmp, tb, db, (long long)E, 0, (int)(2 * sbits), st) != cudaSuccess) {
            rc = WEDGE_ERR_CUDA;
        } else {
            if (E)
                unpack_keys_kernel<<<grid_of(E, 152), 256, 0, st>>>(db.Current(), E, sbits, WEDGE_WEIGHTS_NONE, ds, dd,
                                                                    nullptr);
            if (cudaMemcpy(src, ds, E * sizeof(uint32_t), cudaMemcpyDeviceToHost) != cudaSuccess ||
                cudaMemcpy(dst, dd, E * sizeof(uint32_t), cudaMemcpyDeviceToHost) != cudaSuccess)
                rc = WEDGE_ERR_CUDA;
        }
    }
    cudaFree(tmp);
    cudaFree(alt);
    cudaFree(ds);
    cudaFree(dd);
    cudaFree(keys);
    return rc;
}

int wedge_cuda_rmat_edge_list(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                              int symmetrise, uint64_t* V, uint64_t* E, uint32_t* src, uint32_t* dst, uint64_t capacity)
{
    if (!V || !E || scale < 1 || scale > 31 || edge_factor == 0 || a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
        return WEDGE_ERR_ARG;
    const uint64_t E0 = (uint64_t)edge_factor << scale;
    *V = 1ull << scale;
    *E = symmetrise ? 2 * E0 : E0;
    if (!src)
        return WEDGE_OK;
    if (!dst || capacity < *E)
        return WEDGE_ERR_ARG;
    unsigned long long* keys = nullptr;
    if (cudaMalloc((void**)&keys, *E * sizeof(unsigned long long)) != cudaSuccess)
        return WEDGE_ERR_OOM;
    const unsigned long long ta = (unsigned long long)(a * 4294967296.0);
    const unsigned long long tab = (unsigned long long)((a + b) * 4294967296.0);
    const unsigned long long tabc = (unsigned long long)((a + b + c) * 4294967296.0);
    rmat_kernel<<<grid_of(E0, 152), 256>>>(scale, ta, tab, tabc, seed, E0, symmetrise ? 1 : 0, scale, keys);
    return keys_to_host(keys, *E, scale, src, dst);
}

int wedge_cuda_grid_edge_list(uint32_t side, double long_range_frac, uint64_t seed, uint64_t* V, uint64_t* E,
                              uint32_t* src, uint32_t* dst, uint64_t capacity)
{
    if (!V || !E || side < 2 || side > 65535 || long_range_frac < 0.0)
        return WEDGE_ERR_ARG;
    const uint64_t base = 4ull * side * (side - 1ull);
    const uint64_t lr = (uint64_t)(long_range_frac * (double)base);
    *V = (uint64_t)side * side;
    *E = base + lr;
    if (!src)
        return WEDGE_OK;
    if (!dst || capacity < *E)
        return WEDGE_ERR_ARG;
    const uint32_t sbits = bits_for(*V);
    unsigned long long* keys = nullptr;
    if (cudaMalloc((void**)&keys, *E * sizeof(unsigned long long)) != cudaSuccess)
        return WEDGE_ERR_OOM;
    grid_kernel<<<grid_of(*E, 152), 256>>>(side, lr, seed, sbits, keys);
    return keys_to_host(keys, *E, sbits, src, dst);
}

}  // extern "C"
