// Batched BFS / SSSP queries over many graphs in one persistent cooperative
// kernel (no counterpart in the reference, which runs one query per process).
//
// Every round of the kernel advances every unfinished query by one iteration:
//   build   Wedge frontier of the queries whose next pull is sparse: the
//           out-edge chunks of the vertices the last pull activated are
//           marked (wedge.c:63-155), and newly marked chunks are appended to
//           the query's chunk list -- or, on graphs whose CSRI holds in-edge
//           positions, every activated vertex's out-list becomes PIECE-entry
//           items whose in-edges the pull relaxes one by one (as the single-
//           query engine's SSSP Wedge pulls); the previous frontier bitmaps
//           are cleared
//   prefix  (block 0) per-query chunk counts -> one offset table: the work
//           queue of the pull
//   pull    warps take items from the queue, across all queries, and pull
//           them (phase_edge_pull_bfs.c / _sssp.c logic: gather,
//           per-destination min, the property, activation bit, activated-
//           vertex list, changed out-edge mass): dense pulls in tiles of 256
//           in-edges, sparse ones in marked 32-edge chunks or out-list pieces
//   decide  (block 0) per query: done when no mass changed, else the plain
//           rule (mass > t% of the query's edges: dense) picks the next pull
// with a grid-wide barrier between the phases.  All blocks leave the loop
// together: the exit flag is written by block 0 before a barrier and read by
// every block after it.
#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>

#include "engine.cuh"
#include "pull.cuh"

namespace cg = cooperative_groups;

namespace wedge {

constexpr int BT = 256;                       // threads per persistent block
constexpr uint32_t BATCH_MAX_ROUNDS = 1u << 20; // iteration cap of the slowest query

struct BGraph {
    const uint32_t* src;
    const unsigned long long* w;
    const uint32_t* dst_id;
    const unsigned long long* dst_off;
    const uint32_t* chunk_dst0;  // [nchunks+1] compressed destination owning edge 32*c (Vne past the end)
    const uint32_t* dst_start;   // destination-start bitmap and 128-edge tile index of the graph handle
    const uint32_t* tile_dst0;
    const uint8_t* w8;           // byte-wide weights, or null
    const uint32_t* outdeg;
    const unsigned long long* csri_off;
    const uint32_t* csri;
    uint32_t csri_shift;  // chunk of a CSRI entry: entry >> csri_shift (5: positions, 0: chunk ids)
    const uint32_t* new2old;
    const uint32_t* old2new;
    uint64_t V, E;
    uint32_t Vne, nchunks, weight_kind;
    uint32_t push;               // sparse pulls relax in-edge positions (CSRI of positions)
};

struct BQuery {
    uint32_t graph, app, root_in, pad;
    unsigned long long* prop; // [V] BFS parent (engine id; the root holds itself) / SSSP distance
    uint32_t* front[2];       // [V/32+1] activation bitmaps, current = front[parity]
    uint32_t* list[2];        // [V] the same vertices as lists
    uint32_t* chunk_bits;     // [nchunks/32+1] Wedge frontier
    uint32_t* chunk_list;     // [nchunks] its marked chunks
    uint2* vitems;            // [V + E/PIECE + 1] (vertex, piece) items of a sparse pull over in-edge positions
};

struct BCtl {
    unsigned long long mass;
    uint32_t nlist[2];
    uint32_t items; // chunks of the next pull
    uint32_t mode;
    uint32_t parity;
    uint32_t iter;
    uint32_t done;
    uint32_t root; // engine id
};

struct BShared {
    uint32_t active;
    uint32_t rounds;
    unsigned long long grab_pull, grab_build, grab_clear;
    unsigned long long chunks_pulled;
};

struct BArgs {
    const BGraph* graphs;
    const BQuery* q;
    BCtl* ctl;
    BShared* sh;
    unsigned long long* pull_off;  // [Q+1]
    unsigned long long* build_off; // [Q+1]
    unsigned long long* clear_off; // [Q+1]
    uint32_t Q, threshold_pct, grab, split, max_rounds, pad;
};

__device__ __forceinline__ uint32_t find_owner(const unsigned long long* off, uint32_t Q, unsigned long long i)
{
    // last q with off[q] <= i (off[0] = 0, off[Q] > i)
    uint32_t lo = 0, hi = Q;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (off[mid] <= i)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// exclusive prefix of f(q) over q < Q into off[0..Q] by the threads of one block
template <class F>
__device__ void block_prefix(unsigned long long* off, uint32_t Q, F f)
{
    __shared__ unsigned long long part[BT];
    const uint32_t per = (Q + BT - 1) / BT;
    const uint32_t q0 = threadIdx.x * per, q1 = min(Q, q0 + per);
    unsigned long long s = 0;
    for (uint32_t q = q0; q < q1; ++q)
        s += f(q);
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long run = 0;
        for (int t = 0; t < BT; ++t) {
            const unsigned long long x = part[t];
            part[t] = run;
            run += x;
        }
        off[Q] = run;
    }
    __syncthreads();
    unsigned long long run = part[threadIdx.x];
    for (uint32_t q = q0; q < q1; ++q) {
        off[q] = run;
        run += f(q);
    }
    __syncthreads();
}

__device__ __forceinline__ void mark_batch_chunk(const BQuery& qq, BCtl& c, uint32_t ch)
{
    const uint32_t bit = 1u << (ch & 31u);
    if (!(qq.chunk_bits[ch >> 5] & bit)) {
        const uint32_t old = atomicOr(&qq.chunk_bits[ch >> 5], bit);
        if (!(old & bit)) {
            const uint32_t pos = atomicAdd(&c.items, 1u);
            qq.chunk_list[pos] = ch;
        }
    }
}

// ---------------------------------------------------------------- build (+ clear)
__device__ void phase_build(const BArgs& a)
{
    const int lane = threadIdx.x & 31;
    const unsigned long long total = a.build_off[a.Q];
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0)
            base = atomicAdd(&a.sh->grab_build, 32ull);
        base = __shfl_sync(FULL, base, 0);
        if (base >= total)
            break;
        const unsigned long long i = base + (unsigned long long)lane;
        const bool valid = i < total;
        uint32_t q = 0, v = 0;
        unsigned long long start = 0, len = 0;
        if (valid) {
            q = find_owner(a.build_off, a.Q, i);
            const BCtl& c = a.ctl[q];
            v = a.q[q].list[c.parity][i - a.build_off[q]];
            const BGraph& G = a.graphs[a.q[q].graph];
            start = G.csri_off[v];
            len = G.csri_off[v + 1] - start;
        }
        // sparse pulls over in-edge positions: PIECE-entry items of each out-list
        if (valid && a.graphs[a.q[q].graph].push) {
            const uint32_t np = (uint32_t)((len + PIECE - 1) / PIECE);
            if (np) {
                const uint32_t pos = atomicAdd(&a.ctl[q].items, np);
                for (uint32_t j = 0; j < np; ++j)
                    a.q[q].vitems[pos + j] = make_uint2(v, j);
            }
            len = 0; /* nothing to mark */
        }
        // short lists: one lane each
        if (valid && len <= a.split) {
            const BGraph& G = a.graphs[a.q[q].graph];
            for (unsigned long long j = 0; j < len; ++j)
                mark_batch_chunk(a.q[q], a.ctl[q], G.csri[start + j] >> G.csri_shift);
        }
        // long lists: the whole warp, one list at a time
        uint32_t longs = __ballot_sync(FULL, valid && len > a.split && !a.graphs[a.q[q].graph].push);
        while (longs) {
            const int l = __ffs(longs) - 1;
            longs &= longs - 1u;
            const uint32_t lq = __shfl_sync(FULL, q, l);
            const unsigned long long ls = __shfl_sync(FULL, start, l), ll = __shfl_sync(FULL, len, l);
            const BGraph& G = a.graphs[a.q[lq].graph];
            for (unsigned long long j = lane; j < ll; j += 32)
                mark_batch_chunk(a.q[lq], a.ctl[lq], G.csri[ls + j] >> G.csri_shift);
        }
    }
    // clear the previous frontier bits (their list is exact)
    const unsigned long long ctotal = a.clear_off[a.Q];
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0)
            base = atomicAdd(&a.sh->grab_clear, 32ull);
        base = __shfl_sync(FULL, base, 0);
        if (base >= ctotal)
            break;
        const unsigned long long i = base + (unsigned long long)lane;
        if (i < ctotal) {
            const uint32_t q = find_owner(a.clear_off, a.Q, i);
            const uint32_t old = a.ctl[q].parity ^ 1u;
            const uint32_t v = a.q[q].list[old][i - a.clear_off[q]];
            atomicAnd(&a.q[q].front[old][v >> 5], ~(1u << (v & 31u)));
        }
    }
}

// ---------------------------------------------------------------- prefix (block 0)
__device__ void phase_prefix(const BArgs& a)
{
    block_prefix(a.pull_off, a.Q, [&](uint32_t q) -> unsigned long long {
        const BCtl& c = a.ctl[q];
        return c.done ? 0ull : (unsigned long long)c.items;
    });
    __shared__ uint32_t act;
    if (threadIdx.x == 0)
        act = 0u;
    __syncthreads();
    for (uint32_t q = threadIdx.x; q < a.Q; q += blockDim.x) {
        BCtl& c = a.ctl[q];
        c.nlist[c.parity ^ 1u] = 0u; /* its bits were cleared in the build phase */
        if (!c.done)
            atomicAdd(&act, 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        a.sh->grab_pull = 0ull;
        a.sh->active = act;
        if (act)
            a.sh->rounds += 1u;
    }
}

// ---------------------------------------------------------------- pull
__device__ void pull_chunk(const BArgs& a, uint32_t q, uint32_t ch, uint32_t* heads, unsigned long long& mass)
{
    const int lane = threadIdx.x & 31;
    const BQuery& qq = a.q[q];
    BCtl& c = a.ctl[q];
    const BGraph& G = a.graphs[qq.graph];
    const unsigned long long p = 32ull * ch + (unsigned long long)lane;
    const bool valid = p < G.E;
    const uint32_t s = valid ? G.src[p] : NONE32;
    DevGraph dg;
    dg.Vne = G.Vne;
    dg.dst_off = G.dst_off;
    TileGeo<1> tg;
    tile_geometry<1>(dg, 32ull * ch, ch + 1u >= G.nchunks, G.chunk_dst0[ch], G.chunk_dst0[ch + 1], lane, heads, tg,
                     [](uint32_t, uint32_t) {});
    const uint32_t k = pos_dst(tg, 0);
    const uint32_t* cur = qq.front[c.parity];
    uint32_t* nxt = qq.front[c.parity ^ 1u];
    uint32_t* nlist = qq.list[c.parity ^ 1u];
    auto activate = [&](uint32_t vtx) {
        const uint32_t b = 1u << (vtx & 31u);
        if (!(atomicOr(&nxt[vtx >> 5], b) & b)) {
            const uint32_t pos = atomicAdd(&c.nlist[c.parity ^ 1u], 1u);
            nlist[pos] = vtx;
            mass += G.outdeg[vtx];
        }
    };
    if (qq.app == WEDGE_APP_BFS) {
        uint32_t v[1];
        v[0] = NONE32;
        if (valid && ((cur[s >> 5] >> (s & 31u)) & 1u)) {
            const uint32_t vtx = G.dst_id[k];
            if (qq.prop[vtx] == NONE64) /* unvisited */
                v[0] = s;
        }
        seg_reduce<1>(v, tg, lane, MinU32(), [&](uint32_t kk, uint32_t val, int) {
            if (val == NONE32)
                return;
            const uint32_t vtx = G.dst_id[kk];
            if (atomicMin(&qq.prop[vtx], (unsigned long long)val) == NONE64)
                activate(vtx);
        });
    } else {
        unsigned long long v[1];
        v[0] = NONE64;
        if (valid) {
            const unsigned long long d = qq.prop[s];
            const unsigned long long wt = G.w[p];
            if (G.weight_kind == WEDGE_WEIGHTS_F64)
                v[0] = (unsigned long long)__double_as_longlong(
                    __dadd_rn(__longlong_as_double((long long)d), __longlong_as_double((long long)wt)));
            else
                v[0] = (d == NONE64) ? NONE64 : d + wt; /* phase_edge_pull_sssp.c:136-137 */
        }
        seg_reduce<1>(v, tg, lane, MinU64(), [&](uint32_t kk, unsigned long long val, int) {
            if (val == NONE64)
                return;
            const uint32_t vtx = G.dst_id[kk];
            if (val < qq.prop[vtx] && val < atomicMin(&qq.prop[vtx], val))
                activate(vtx);
        });
    }
}

// A dense pull's item: a tile of BTILE_CH chunks (32*BEPL in-edges), lane l
// holding BEPL consecutive ones, with the single-query engine's tile machinery
// (destination-start bitmap geometry, segmented reduction).  BFS gathers the
// frontier bits of the sources and claims an unvisited destination for the
// least frontier source with one compare-and-swap; SSSP gathers distances,
// adds the weights and lowers the destination with atomicMin.  Per
// destination, not per in-edge: the visited test, the property write and the
// activation.
constexpr int BEPL = 8;
constexpr uint32_t BTILE_CH = BEPL; /* 32-edge chunks per tile */

__device__ void pull_tile(const BArgs& a, uint32_t q, uint32_t t, unsigned long long& mass)
{
    const int lane = threadIdx.x & 31;
    const BQuery& qq = a.q[q];
    BCtl& c = a.ctl[q];
    const BGraph& G = a.graphs[qq.graph];
    const uint64_t base = (uint64_t)t * (32u * BEPL);
    const uint32_t ch0 = t * BTILE_CH;
    const uint32_t k0 = G.chunk_dst0[ch0];
    const uint32_t kend = G.chunk_dst0[min(ch0 + BTILE_CH, G.nchunks)];
    const bool last = base + 32u * BEPL >= G.E;
    uint32_t sa[BEPL];
    {
        const uint64_t p0 = base + (uint64_t)lane * BEPL;
        uint32_t x[8];
        ld_stream_v8(G.src + p0, x);
#pragma unroll
        for (int j = 0; j < BEPL; ++j)
            sa[j] = (p0 + (uint64_t)j < G.E) ? x[j] : NONE32;
    }
    DevGraph dg;
    dg.dst_start = G.dst_start;
    TileGeo<BEPL> tg;
    const uint32_t* cur = qq.front[c.parity];
    uint32_t* nxt = qq.front[c.parity ^ 1u];
    uint32_t* nlist = qq.list[c.parity ^ 1u];
    auto activate = [&](uint32_t vtx) {
        const uint32_t b = 1u << (vtx & 31u);
        if (!(atomicOr(&nxt[vtx >> 5], b) & b)) {
            const uint32_t pos = atomicAdd(&c.nlist[c.parity ^ 1u], 1u);
            nlist[pos] = vtx;
            mass += G.outdeg[vtx];
        }
    };
    if (qq.app == WEDGE_APP_BFS) {
        uint32_t v[BEPL];
#pragma unroll
        for (int j = 0; j < BEPL; ++j) {
            const uint32_t x = sa[j];
            v[j] = (x != NONE32 && ((cur[x >> 5] >> (x & 31u)) & 1u)) ? x : NONE32;
        }
        tile_geometry_bits<BEPL>(dg, base, last, k0, kend, lane, tg);
        seg_reduce<BEPL>(v, tg, lane, MinU32(), [&](uint32_t k, uint32_t val, int) {
            if (val == NONE32)
                return;
            const uint32_t vtx = G.dst_id[k];
            /* the least frontier source of this tile claims an unvisited destination */
            if (qq.prop[vtx] == NONE64 && atomicCAS(&qq.prop[vtx], NONE64, (unsigned long long)val) == NONE64)
                activate(vtx);
        });
    } else {
        const bool f64 = G.weight_kind == WEDGE_WEIGHTS_F64;
        unsigned long long v[BEPL];
        const uint64_t p0 = base + (uint64_t)lane * BEPL;
#pragma unroll
        for (int j = 0; j < BEPL; ++j) {
            const uint32_t x = sa[j];
            v[j] = NONE64;
            if (x != NONE32) {
                const unsigned long long d = qq.prop[x];
                const unsigned long long wt = G.w8 ? (unsigned long long)G.w8[p0 + j] : G.w[p0 + j];
                if (f64)
                    v[j] = (unsigned long long)__double_as_longlong(
                        __dadd_rn(__longlong_as_double((long long)d), __longlong_as_double((long long)wt)));
                else
                    v[j] = (d == NONE64) ? NONE64 : d + wt; /* phase_edge_pull_sssp.c:136-137 */
            }
        }
        tile_geometry_bits<BEPL>(dg, base, last, k0, kend, lane, tg);
        seg_reduce<BEPL>(v, tg, lane, MinU64(), [&](uint32_t k, unsigned long long val, int) {
            if (val == NONE64)
                return;
            const uint32_t vtx = G.dst_id[k];
            if (val < qq.prop[vtx] && val < atomicMin(&qq.prop[vtx], val))
                activate(vtx);
        });
    }
}

// A sparse pull over in-edge positions: the in-edges of one PIECE of an
// activated vertex's out-list are relaxed by the warp's lanes (BFS: an
// unvisited destination takes the vertex as its parent; SSSP: min-plus)
__device__ void push_piece(const BArgs& a, uint32_t q, uint2 it, unsigned long long& mass)
{
    const int lane = threadIdx.x & 31;
    const BQuery& qq = a.q[q];
    BCtl& c = a.ctl[q];
    const BGraph& G = a.graphs[qq.graph];
    uint32_t* nxt = qq.front[c.parity ^ 1u];
    uint32_t* nlist = qq.list[c.parity ^ 1u];
    auto activate = [&](uint32_t vtx) {
        const uint32_t b = 1u << (vtx & 31u);
        if (!(atomicOr(&nxt[vtx >> 5], b) & b)) {
            const uint32_t pos = atomicAdd(&c.nlist[c.parity ^ 1u], 1u);
            nlist[pos] = vtx;
            mass += G.outdeg[vtx];
        }
    };
    const unsigned long long lo = G.csri_off[it.x] + (unsigned long long)it.y * PIECE;
    const unsigned long long end = G.csri_off[it.x + 1u];
    const unsigned long long hi = (lo + PIECE < end) ? lo + PIECE : end;
    const unsigned long long du = qq.prop[it.x];
    const bool f64 = G.weight_kind == WEDGE_WEIGHTS_F64;
    for (unsigned long long j = lo + (unsigned long long)lane; j < hi; j += 32u) {
        const uint32_t p = G.csri[j];
        const uint32_t vtx = G.dst_id[dst_of_pos(G.dst_start, G.tile_dst0, p)];
        if (qq.app == WEDGE_APP_BFS) {
            if (qq.prop[vtx] == NONE64 && atomicCAS(&qq.prop[vtx], NONE64, (unsigned long long)it.x) == NONE64)
                activate(vtx);
        } else {
            const unsigned long long wt = G.w8 ? (unsigned long long)G.w8[p] : G.w[p];
            const unsigned long long nd =
                f64 ? (unsigned long long)__double_as_longlong(
                          __dadd_rn(__longlong_as_double((long long)du), __longlong_as_double((long long)wt)))
                    : du + wt; /* phase_edge_pull_sssp.c:136-137; an activated source is reached */
            if (nd < qq.prop[vtx] && nd < atomicMin(&qq.prop[vtx], nd))
                activate(vtx);
        }
    }
}

__device__ void phase_pull(const BArgs& a)
{
    __shared__ uint32_t heads_all[BT / 32];
    const int lane = threadIdx.x & 31;
    uint32_t* heads = &heads_all[threadIdx.x >> 5];
    const unsigned long long total = a.pull_off[a.Q];
    unsigned long long pulled = 0;
    uint32_t q = 0;
    for (;;) {
        unsigned long long base = 0;
        if (lane == 0)
            base = atomicAdd(&a.sh->grab_pull, (unsigned long long)a.grab);
        base = __shfl_sync(FULL, base, 0);
        if (base >= total)
            break;
        const unsigned long long end = min(total, base + a.grab);
        for (unsigned long long i = base; i < end; ++i) {
            if (!(a.pull_off[q] <= i && i < a.pull_off[q + 1]))
                q = find_owner(a.pull_off, a.Q, i); /* warp-uniform */
            const unsigned long long local = i - a.pull_off[q];
            const BCtl& c = a.ctl[q];
            const bool sparse = c.mode == MODE_WEDGE;
            const bool push = sparse && a.graphs[a.q[q].graph].push;
            const uint32_t ch = (sparse && !push) ? a.q[q].chunk_list[local] : (uint32_t)local;
            unsigned long long mass = 0;
            if (push)
                push_piece(a, q, a.q[q].vitems[local], mass);
            else if (sparse)
                pull_chunk(a, q, ch, heads, mass);
            else
                pull_tile(a, q, (uint32_t)local, mass); /* dense: tiles of BTILE_CH chunks */
#pragma unroll
            for (int d = 16; d > 0; d >>= 1)
                mass += __shfl_xor_sync(FULL, mass, d);
            if (lane == 0) {
                if (mass)
                    atomicAdd(&a.ctl[q].mass, mass);
                if (sparse && !push)
                    atomicAnd(&a.q[q].chunk_bits[ch >> 5], ~(1u << (ch & 31u))); /* consumed */
            }
            ++pulled;
        }
    }
    if (lane == 0 && pulled)
        atomicAdd(&a.sh->chunks_pulled, pulled);
}

// ---------------------------------------------------------------- decide (block 0)
__device__ void phase_decide(const BArgs& a)
{
    for (uint32_t q = threadIdx.x; q < a.Q; q += blockDim.x) {
        BCtl& c = a.ctl[q];
        if (c.done)
            continue;
        const BGraph& G = a.graphs[a.q[q].graph];
        c.iter += 1u;
        const unsigned long long m = c.mass;
        c.mass = 0ull;
        if (m == 0ull || c.iter >= a.max_rounds) { /* execution_bfs.c:239-251 */
            c.done = 1u;
            continue;
        }
        c.parity ^= 1u;
        const unsigned long long thr = (G.E * (unsigned long long)a.threshold_pct) / 100ull; /* execution_bfs.c:132 */
        c.mode = m > thr ? MODE_DENSE : MODE_WEDGE;                                         /* execution_bfs.c:141 */
        c.items = c.mode == MODE_DENSE ? (G.nchunks + BTILE_CH - 1u) / BTILE_CH : 0u;
    }
    __syncthreads();
    block_prefix(a.build_off, a.Q, [&](uint32_t q) -> unsigned long long {
        const BCtl& c = a.ctl[q];
        return (!c.done && c.mode == MODE_WEDGE) ? (unsigned long long)c.nlist[c.parity] : 0ull;
    });
    block_prefix(a.clear_off, a.Q, [&](uint32_t q) -> unsigned long long {
        const BCtl& c = a.ctl[q];
        return c.done ? 0ull : (unsigned long long)c.nlist[c.parity ^ 1u];
    });
    if (threadIdx.x == 0) {
        a.sh->grab_build = 0ull;
        a.sh->grab_clear = 0ull;
    }
}

__global__ void __launch_bounds__(BT) batch_kernel(BArgs a)
{
    cg::grid_group grid = cg::this_grid();
    for (uint32_t round = 0; round < a.max_rounds + 1u; ++round) {
        phase_build(a);
        grid.sync();
        if (blockIdx.x == 0)
            phase_prefix(a);
        grid.sync();
        if (*(volatile uint32_t*)&a.sh->active == 0u) /* written before the barrier, uniform after it */
            break;
        phase_pull(a);
        grid.sync();
        if (blockIdx.x == 0)
            phase_decide(a);
        grid.sync();
    }
}

// ---------------------------------------------------------------- setup kernels
__global__ void batch_chunk_index_kernel(BGraph G, uint32_t* chunk_dst0)
{
    // chunk_dst0[c] = compressed destination owning edge 32c: last k with dst_off[k] <= 32c
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c <= G.nchunks; c += gridDim.x * blockDim.x) {
        const unsigned long long p = 32ull * c;
        uint32_t k;
        if (p >= G.E) {
            k = G.Vne;
        } else {
            uint32_t lo = 0, hi = G.Vne;
            while (hi - lo > 1u) {
                const uint32_t mid = (lo + hi) >> 1;
                if (G.dst_off[mid] <= p)
                    lo = mid;
                else
                    hi = mid;
            }
            k = lo;
        }
        chunk_dst0[c] = k;
    }
}

__global__ void batch_reset_kernel(const BGraph* graphs, const BQuery* qs, uint32_t Q)
{
    const uint32_t q = blockIdx.y;
    if (q >= Q)
        return;
    const BQuery& qq = qs[q];
    const BGraph& G = graphs[qq.graph];
    const unsigned long long inf = (qq.app == WEDGE_APP_SSSP && G.weight_kind == WEDGE_WEIGHTS_F64)
                                       ? 0x7FF0000000000000ull /* execution_sssp.c:78, as double */
                                       : NONE64;
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    for (uint64_t v = t0; v < G.V; v += stride)
        qq.prop[v] = inf;
    for (uint64_t i = t0; i < (G.V + 31) / 32 + 1; i += stride) {
        qq.front[0][i] = 0u;
        qq.front[1][i] = 0u;
    }
    for (uint64_t i = t0; i < (uint64_t)G.nchunks / 32 + 1; i += stride)
        qq.chunk_bits[i] = 0u;
}

__global__ void batch_seed_kernel(BArgs a)
{
    // roots (execution_bfs.c:110-117, execution_sssp.c:83-88), first modes, first offsets
    for (uint32_t q = threadIdx.x; q < a.Q; q += blockDim.x) {
        const BQuery& qq = a.q[q];
        const BGraph& G = a.graphs[qq.graph];
        BCtl& c = a.ctl[q];
        const uint32_t root_in = qq.root_in < G.V ? qq.root_in : 0u; /* main.c:81-85 */
        const uint32_t r = G.old2new[root_in];
        c.root = r;
        c.mass = 0ull;
        c.parity = 0u;
        c.iter = 0u;
        c.done = G.E == 0ull ? 1u : 0u;
        qq.prop[r] = (qq.app == WEDGE_APP_BFS) ? (unsigned long long)r : 0ull;
        qq.front[0][r >> 5] |= 1u << (r & 31u);
        qq.list[0][0] = r;
        c.nlist[0] = 1u;
        c.nlist[1] = 0u;
        const unsigned long long thr = (G.E * (unsigned long long)a.threshold_pct) / 100ull;
        c.mode = (unsigned long long)G.outdeg[r] > thr ? MODE_DENSE : MODE_WEDGE;
        c.items = c.mode == MODE_DENSE ? (G.nchunks + BTILE_CH - 1u) / BTILE_CH : 0u;
    }
    __syncthreads();
    block_prefix(a.build_off, a.Q, [&](uint32_t q) -> unsigned long long {
        const BCtl& c = a.ctl[q];
        return (!c.done && c.mode == MODE_WEDGE) ? 1ull : 0ull;
    });
    block_prefix(a.clear_off, a.Q, [&](uint32_t) -> unsigned long long { return 0ull; });
    if (threadIdx.x == 0) {
        a.sh->active = 0u;
        a.sh->rounds = 0u;
        a.sh->grab_pull = a.sh->grab_build = a.sh->grab_clear = 0ull;
        a.sh->chunks_pulled = 0ull;
    }
}

__global__ void batch_export_kernel(BGraph G, BQuery qq, uint32_t root, unsigned long long* out)
{
    for (uint64_t o = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; o < G.V; o += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t v = G.old2new[o];
        const unsigned long long x = qq.prop[v];
        if (qq.app == WEDGE_APP_BFS)
            out[o] = (x == NONE64 || v == root) ? NONE64 : (unsigned long long)G.new2old[(uint32_t)x];
        else
            out[o] = x;
    }
}

}  // namespace wedge

using namespace wedge;

static uint32_t bgrid(uint64_t work, uint32_t threads, uint32_t cap)
{
    const uint64_t g = (work + threads - 1) / threads;
    return (uint32_t)(g == 0 ? 1 : (g < cap ? g : cap));
}

struct wedge_batch {
    int device;
    int num_sms;
    cudaStream_t stream;
    cudaEvent_t ev[2];
    uint32_t Q, G;
    BGraph* d_graphs;
    BQuery* d_queries;
    BCtl* d_ctl;
    BShared* d_sh;
    unsigned long long* d_off; // 3 * (Q+1)
    BGraph* h_graphs;
    BQuery* h_queries;
    void* allocs[16];
    int nallocs;
    void** qallocs; // per-query buffers
    uint32_t nq_allocs;
    cudaGraphExec_t exec;
    wedge_batch_tuning_t exec_tuning;
    uint32_t exec_blocks;
};

static void batch_release(wedge_batch* b)
{
    if (!b)
        return;
    if (b->stream)
        cudaStreamSynchronize(b->stream);
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    for (int i = 0; i < b->nallocs; ++i)
        cudaFree(b->allocs[i]);
    for (uint32_t i = 0; i < b->nq_allocs; ++i)
        cudaFree(b->qallocs[i]);
    free(b->qallocs);
    free(b->h_graphs);
    free(b->h_queries);
    for (int i = 0; i < 2; ++i)
        if (b->ev[i])
            cudaEventDestroy(b->ev[i]);
    if (b->stream)
        cudaStreamDestroy(b->stream);
    free(b);
}

template <class T>
static int balloc(wedge_batch* b, T** p, uint64_t count, bool per_query)
{
    *p = nullptr;
    const cudaError_t e = cudaMalloc((void**)p, (size_t)(count ? count : 1) * sizeof(T));
    if (e != cudaSuccess)
        return cuda_status(e);
    if (per_query)
        b->qallocs[b->nq_allocs++] = *p;
    else
        b->allocs[b->nallocs++] = *p;
    return WEDGE_OK;
}

extern "C" int wedge_cuda_batch_create(wedge_graph_t* const* graphs, uint32_t num_graphs, const wedge_query_t* queries,
                                       uint32_t num_queries, wedge_batch_t** out)
{
    if (!out || !graphs || !queries || num_graphs == 0 || num_queries == 0 || num_queries > 65535u)
        return WEDGE_ERR_ARG; /* one grid row per query in the reset kernel */
    *out = nullptr;
    const int dev = graphs[0] ? graphs[0]->device : -1;
    for (uint32_t i = 0; i < num_graphs; ++i)
        if (!graphs[i] || graphs[i]->device != dev || graphs[i]->g.V > 0xFFFFFFFEull)
            return WEDGE_ERR_ARG;
    for (uint32_t i = 0; i < num_queries; ++i) {
        const wedge_query_t& q = queries[i];
        if (q.graph >= num_graphs || (q.app != WEDGE_APP_BFS && q.app != WEDGE_APP_SSSP))
            return WEDGE_ERR_ARG;
        if (q.app == WEDGE_APP_SSSP && graphs[q.graph]->weight_kind == WEDGE_WEIGHTS_NONE)
            return WEDGE_ERR_ARG; /* SSSP needs a weighted load (application.c:171) */
    }
    WEDGE_CHECK(cudaSetDevice(dev));
    wedge_batch* b = (wedge_batch*)calloc(1, sizeof(wedge_batch));
    if (!b)
        return WEDGE_ERR_OOM;
    b->device = dev;
    b->Q = num_queries;
    b->G = num_graphs;
    b->qallocs = (void**)calloc((size_t)num_queries * 8 + num_graphs + 1, sizeof(void*)); /* 8 arrays per query */
    b->h_graphs = (BGraph*)calloc(num_graphs, sizeof(BGraph));
    b->h_queries = (BQuery*)calloc(num_queries, sizeof(BQuery));
    int rc = WEDGE_OK;
    auto fail = [&](int r) {
        batch_release(b);
        return r;
    };
    if (!b->qallocs || !b->h_graphs || !b->h_queries)
        return fail(WEDGE_ERR_OOM);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&b->ev[0]) != cudaSuccess || cudaEventCreate(&b->ev[1]) != cudaSuccess ||
        cudaDeviceGetAttribute(&b->num_sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return fail(WEDGE_ERR_CUDA);
    for (uint32_t i = 0; i < num_graphs; ++i) {
        const DevGraph& g = graphs[i]->g;
        BGraph& G = b->h_graphs[i];
        G.src = g.src;
        G.w = g.w;
        G.dst_id = g.dst_id;
        G.dst_off = g.dst_off;
        G.outdeg = g.outdeg;
        G.csri_off = g.csri_off;
        G.csri = g.csri;
        G.csri_shift = g.csri_pos ? 5u : 0u;
        G.push = g.csri_pos ? 1u : 0u;
        G.dst_start = g.dst_start;
        G.tile_dst0 = g.tile_dst0;
        G.w8 = g.w8;
        G.new2old = g.new2old;
        G.old2new = g.old2new;
        G.V = g.V;
        G.E = g.E;
        G.Vne = g.Vne;
        G.nchunks = (uint32_t)((g.E + 31) / 32);
        G.weight_kind = g.weight_kind;
        uint32_t* cd = nullptr;
        if ((rc = balloc(b, &cd, (uint64_t)G.nchunks + 1, true)))
            return fail(rc);
        G.chunk_dst0 = cd;
        batch_chunk_index_kernel<<<bgrid((uint64_t)G.nchunks + 1, 256, (uint32_t)b->num_sms * 8), 256, 0, b->stream>>>(G, cd);
    }
    for (uint32_t i = 0; i < num_queries; ++i) {
        const BGraph& G = b->h_graphs[queries[i].graph];
        BQuery& q = b->h_queries[i];
        q.graph = queries[i].graph;
        q.app = (uint32_t)queries[i].app;
        q.root_in = queries[i].root < G.V ? (uint32_t)queries[i].root : 0u;
        const uint64_t words = (G.V + 31) / 32 + 1;
        if ((rc = balloc(b, &q.prop, G.V, true)) || (rc = balloc(b, &q.front[0], words, true)) ||
            (rc = balloc(b, &q.front[1], words, true)) || (rc = balloc(b, &q.list[0], G.V, true)) ||
            (rc = balloc(b, &q.list[1], G.V, true)) || (rc = balloc(b, &q.chunk_bits, (uint64_t)G.nchunks / 32 + 1, true)) ||
            (rc = balloc(b, &q.chunk_list, (uint64_t)G.nchunks, true)) ||
            (rc = balloc(b, &q.vitems, G.push ? G.V + G.E / PIECE + 1 : 1, true)))
            return fail(rc);
    }
    if ((rc = balloc(b, &b->d_graphs, num_graphs, false)) || (rc = balloc(b, &b->d_queries, num_queries, false)) ||
        (rc = balloc(b, &b->d_ctl, num_queries, false)) || (rc = balloc(b, &b->d_sh, 1, false)) ||
        (rc = balloc(b, &b->d_off, 3ull * (num_queries + 1), false)))
        return fail(rc);
    if (cudaMemcpyAsync(b->d_graphs, b->h_graphs, sizeof(BGraph) * num_graphs, cudaMemcpyHostToDevice, b->stream) !=
            cudaSuccess ||
        cudaMemcpyAsync(b->d_queries, b->h_queries, sizeof(BQuery) * num_queries, cudaMemcpyHostToDevice, b->stream) !=
            cudaSuccess ||
        cudaStreamSynchronize(b->stream) != cudaSuccess || cudaGetLastError() != cudaSuccess)
        return fail(WEDGE_ERR_CUDA);
    *out = b;
    return WEDGE_OK;
}

static void batch_tuning_defaults(const wedge_batch_tuning_t* in, int occ, wedge_batch_tuning_t* t)
{
    memset(t, 0, sizeof(*t));
    if (in)
        *t = *in;
    if (t->threshold_pct == 0 || t->threshold_pct > 100)
        t->threshold_pct = 20;
    if (t->grab == 0)
        t->grab = 8;
    if (t->blocks_per_sm == 0 || (int)t->blocks_per_sm > occ)
        t->blocks_per_sm = (uint32_t)occ;
    if (t->split == 0)
        t->split = 32;
}

static int batch_enqueue(wedge_batch* b, const wedge_batch_tuning_t& t, uint32_t blocks)
{
    BArgs a;
    memset(&a, 0, sizeof(a));
    a.graphs = b->d_graphs;
    a.q = b->d_queries;
    a.ctl = b->d_ctl;
    a.sh = b->d_sh;
    a.pull_off = b->d_off;
    a.build_off = b->d_off + (b->Q + 1);
    a.clear_off = b->d_off + 2ull * (b->Q + 1);
    a.Q = b->Q;
    a.threshold_pct = t.threshold_pct;
    a.grab = t.grab;
    a.split = t.split;
    a.max_rounds = BATCH_MAX_ROUNDS;
    dim3 rgrid(64, b->Q);
    batch_reset_kernel<<<rgrid, 256, 0, b->stream>>>(b->d_graphs, b->d_queries, b->Q);
    batch_seed_kernel<<<1, BT, 0, b->stream>>>(a);
    void* args[] = {&a};
    WEDGE_CHECK(cudaLaunchCooperativeKernel((const void*)batch_kernel, dim3(blocks), dim3(BT), args, 0, b->stream));
    return WEDGE_OK;
}

extern "C" int wedge_cuda_batch_run(wedge_batch_t* b, const wedge_batch_tuning_t* tuning, uint32_t flags,
                                    wedge_batch_stats_t* stats)
{
    if (!b)
        return WEDGE_ERR_ARG;
    WEDGE_CHECK(cudaSetDevice(b->device));
    int occ = 0;
    WEDGE_CHECK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, batch_kernel, BT, 0));
    if (occ < 1)
        return WEDGE_ERR_CUDA;
    wedge_batch_tuning_t t;
    batch_tuning_defaults(tuning, occ, &t);
    const uint32_t blocks = (uint32_t)b->num_sms * t.blocks_per_sm;
    bool captured = false;
    WEDGE_CHECK(cudaEventRecord(b->ev[0], b->stream));
    if (flags & WEDGE_FLAG_GRAPH) {
        if (b->exec && memcmp(&b->exec_tuning, &t, sizeof(t)) != 0) {
            cudaGraphExecDestroy(b->exec);
            b->exec = nullptr;
        }
        if (!b->exec) {
            cudaGraph_t graph = nullptr;
            if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
                const int rc = batch_enqueue(b, t, blocks);
                const cudaError_t e = cudaStreamEndCapture(b->stream, &graph);
                if (rc == WEDGE_OK && e == cudaSuccess && graph &&
                    cudaGraphInstantiate(&b->exec, graph, 0) == cudaSuccess) {
                    b->exec_tuning = t;
                    b->exec_blocks = blocks;
                } else {
                    b->exec = nullptr;
                }
                if (graph)
                    cudaGraphDestroy(graph);
            }
            cudaGetLastError(); /* a refused capture falls back to direct launches */
        }
        if (b->exec) {
            WEDGE_CHECK(cudaGraphLaunch(b->exec, b->stream));
            captured = true;
        }
    }
    if (!captured) {
        const int rc = batch_enqueue(b, t, blocks);
        if (rc)
            return rc;
    }
    WEDGE_CHECK(cudaEventRecord(b->ev[1], b->stream));
    WEDGE_CHECK(cudaStreamSynchronize(b->stream));
    WEDGE_CHECK(cudaGetLastError());
    BShared sh;
    WEDGE_CHECK(cudaMemcpy(&sh, b->d_sh, sizeof(sh), cudaMemcpyDeviceToHost));
    if (stats) {
        memset(stats, 0, sizeof(*stats));
        float ms = 0.0f;
        cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]);
        stats->running_ms = ms;
        stats->rounds = sh.rounds;
        stats->chunks_pulled = sh.chunks_pulled;
        stats->captured = captured ? 1u : 0u;
        stats->blocks = blocks;
        BCtl* c = (BCtl*)malloc(sizeof(BCtl) * b->Q);
        if (!c)
            return WEDGE_ERR_OOM;
        cudaError_t e = cudaMemcpy(c, b->d_ctl, sizeof(BCtl) * b->Q, cudaMemcpyDeviceToHost);
        uint64_t it = 0;
        for (uint32_t i = 0; i < b->Q; ++i)
            it += c[i].iter;
        free(c);
        WEDGE_CHECK(e);
        stats->iterations = it;
    }
    return WEDGE_OK;
}

extern "C" int wedge_cuda_batch_read_result(wedge_batch_t* b, uint32_t query, void* host_props, uint64_t bytes)
{
    if (!b || query >= b->Q || !host_props)
        return WEDGE_ERR_ARG;
    const BQuery& q = b->h_queries[query];
    const BGraph& G = b->h_graphs[q.graph];
    if (bytes < 8ull * G.V)
        return WEDGE_ERR_ARG;
    WEDGE_CHECK(cudaSetDevice(b->device));
    BCtl c;
    WEDGE_CHECK(cudaMemcpy(&c, b->d_ctl + query, sizeof(c), cudaMemcpyDeviceToHost));
    unsigned long long* tmp = nullptr;
    WEDGE_CHECK(cudaMallocAsync((void**)&tmp, 8ull * (G.V ? G.V : 1), b->stream));
    batch_export_kernel<<<bgrid(G.V, 256, (uint32_t)b->num_sms * 8), 256, 0, b->stream>>>(G, q, c.root, tmp);
    const cudaError_t e = cudaMemcpyAsync(host_props, tmp, 8ull * G.V, cudaMemcpyDeviceToHost, b->stream);
    cudaFreeAsync(tmp, b->stream);
    WEDGE_CHECK(e);
    WEDGE_CHECK(cudaStreamSynchronize(b->stream));
    return WEDGE_OK;
}

extern "C" int wedge_cuda_batch_iterations(wedge_batch_t* b, uint32_t* host_iterations, uint32_t num_queries)
{
    if (!b || !host_iterations || num_queries < b->Q)
        return WEDGE_ERR_ARG;
    WEDGE_CHECK(cudaSetDevice(b->device));
    BCtl* c = (BCtl*)malloc(sizeof(BCtl) * b->Q);
    if (!c)
        return WEDGE_ERR_OOM;
    const cudaError_t e = cudaMemcpy(c, b->d_ctl, sizeof(BCtl) * b->Q, cudaMemcpyDeviceToHost);
    for (uint32_t i = 0; i < b->Q && e == cudaSuccess; ++i)
        host_iterations[i] = c[i].iter;
    free(c);
    WEDGE_CHECK(e);
    return WEDGE_OK;
}

extern "C" void wedge_cuda_batch_free(wedge_batch_t* b) { batch_release(b); }
