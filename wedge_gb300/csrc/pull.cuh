// Edge-pull building blocks of the sm_103a engine.
//
// One warp owns one tile of 32*EPL consecutive in-edges of the
// destination-grouped CSC at a time: lane l loads its EPL consecutive sources
// (whole 32-byte sectors per lane), gathers the EPL source properties, and the
// warp folds them per destination with a segmented reduction (lane-local runs,
// then a 5-step shuffle scan).  A destination whose in-edges lie inside one
// tile is finished by that warp alone; one that spans tiles (a hub) gets one
// partial per tile, combined with atomicMin for the min-reductions and with a
// fixed-order fixup pass for PageRank sums.  This replaces the reference's
// per-thread vector loops and merge buffers (phase_edge_pull_*.c,
// phases.c:54-114): every destination has exactly one owner per tile, so no
// merge buffer is needed.
#pragma once

#include "engine.cuh"

namespace wedge {

// 256-bit streaming loads (sm_100+): one lane reads a whole 32-byte sector, so
// a warp's strided per-lane runs cost one L2 request per sector and need no
// L1 reuse (the L1 is mostly given to the hub cache)
__device__ __forceinline__ void ld_stream_v8(const uint32_t* p, uint32_t (&r)[8])
{
    asm volatile("ld.global.nc.L1::no_allocate.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "l"(p));
}

// the same with an L2 evict-first policy: the in-edge stream is read once per
// pull and should not push the gathered property array out of L2
__device__ __forceinline__ unsigned long long l2_evict_first_policy()
{
    unsigned long long pol;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}

__device__ __forceinline__ void ld_stream_v8_ef(const uint32_t* p, uint32_t (&r)[8], unsigned long long pol)
{
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8], %9;"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "l"(p), "l"(pol));
}

__device__ __forceinline__ void ld_stream_v4u64(const unsigned long long* p, unsigned long long (&r)[4])
{
    asm volatile("ld.global.nc.L1::no_allocate.v4.u64 {%0,%1,%2,%3}, [%4];"
                 : "=l"(r[0]), "=l"(r[1]), "=l"(r[2]), "=l"(r[3])
                 : "l"(p));
}

__device__ __forceinline__ unsigned long long ld_stream_u64(const void* p)
{
    unsigned long long r;
    asm volatile("ld.global.nc.L1::no_allocate.u64 %0, [%1];" : "=l"(r) : "l"(p));
    return r;
}

// evict-first forms of the streaming loads (weights beside the in-edge sources)
__device__ __forceinline__ unsigned long long ld_stream_u64_ef(const void* p, unsigned long long pol)
{
    unsigned long long r;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.u64 %0, [%1], %2;" : "=l"(r) : "l"(p), "l"(pol));
    return r;
}

__device__ __forceinline__ void ld_stream_v4u64_ef(const unsigned long long* p, unsigned long long (&r)[4],
                                                   unsigned long long pol)
{
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u64 {%0,%1,%2,%3}, [%4], %5;"
                 : "=l"(r[0]), "=l"(r[1]), "=l"(r[2]), "=l"(r[3])
                 : "l"(p), "l"(pol));
}

__device__ __forceinline__ uint4 ld_stream_v4u32_ef(const void* p, unsigned long long pol)
{
    uint4 r;
    asm volatile("ld.global.nc.L1::no_allocate.L2::cache_hint.v4.u32 {%0,%1,%2,%3}, [%4], %5;"
                 : "=r"(r.x), "=r"(r.y), "=r"(r.z), "=r"(r.w)
                 : "l"(p), "l"(pol));
    return r;
}

/* ---- hub cache: a bulk (TMA) copy of the low-id end of the gathered array
 * into shared memory, completed on an mbarrier.  Vertices are relabelled by
 * descending out-degree, so ids [0, hub_n) are the sources most in-edges
 * name; their gathers then hit shared memory instead of L1/L2. */
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(unsigned long long* bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// non-blocking probe of the barrier's phase `parity`
__device__ __forceinline__ bool mbar_test_wait(unsigned long long* bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0u;
}

// bounded wait: false when the phase did not complete within `tries` probes
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, uint32_t parity, uint32_t tries)
{
    for (uint32_t i = 0; i < tries; ++i) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok)
                     : "r"(smem_u32(bar)), "r"(parity)
                     : "memory");
        if (ok)
            return true;
    }
    return false;
}

// global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, unsigned long long* bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

// read-only (non-coherent) path for arrays no kernel writes while it runs
__device__ __forceinline__ uint32_t ld_ro_u32(const uint32_t* p)
{
    uint32_t r;
    asm volatile("ld.global.nc.u32 %0, [%1];" : "=r"(r) : "l"(p));
    return r;
}

__device__ __forceinline__ double ld_ro_f64(const double* p)
{
    double r;
    asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(r) : "l"(p));
    return r;
}

// a gathered 32-bit property that the launch itself may write (no .nc):
// allocating in L1 with evict-last, so that the properties most gathered stay
__device__ __forceinline__ uint32_t ld_gather_u32(const uint32_t* p)
{
    uint32_t r;
    asm volatile("ld.global.L1::evict_last.u32 %0, [%1];" : "=r"(r) : "l"(p));
    return r;
}

__device__ __forceinline__ float ld_ro_f32(const float* p)
{
    float r;
    /* allocating in L1, evict-last: the ranks most gathered stay (0.8% faster per PageRank at R-MAT scale 26
       than the default policy; an L2 evict-last hint measured slower) */
    asm volatile("ld.global.nc.L1::evict_last.f32 %0, [%1];" : "=f"(r) : "l"(p));
    return r;
}

// Per-lane geometry of a tile of TILE_E = 32*EPL consecutive in-edges; lane l
// owns positions [EPL*l, EPL*l + EPL).
template <int EPL>
struct TileGeo {
    uint64_t base;
    uint32_t k0;         // compressed destination of position 0
    uint32_t before;     // destination starts at positions [1, EPL*lane)
    uint32_t nib;        // starts at the lane's EPL positions (bit 0 for lane 0 = k0 starts at base)
    uint32_t nib_inner;  // nib without the lane-0 position-0 marker
    uint32_t ndst;       // destinations with in-edges in this tile
    bool k0_fresh;       // k0 starts exactly at the tile start
    bool tail_cont;      // the tile's last destination continues into the next tile
};

// Destination ranks inside a tile from dst_off (the batched kernel's form):
// position p belongs to compressed destination k0 + (number of destination
// starts in [1, p]).  k0 / kend are the compressed
// destinations owning the tile's first edge and the next tile's first edge.
// The starts are collected in the warp's shared `heads` words (EPL words) and
// prefix-counted with a shuffle scan.  fill(slot, k) is called once for every
// destination k with in-edges in the tile (slot = k - k0, on some lane) so the
// caller can stage per-destination data in shared memory; everything is visible
// after the final __syncwarp.
template <int EPL, class Fill>
__device__ __forceinline__ void tile_geometry(const DevGraph& g, uint64_t base, bool last_tile, uint32_t k0,
                                              uint32_t kend, int lane, uint32_t* heads, TileGeo<EPL>& tg, Fill fill)
{
    constexpr uint32_t TILE_E = 32u * EPL;
    tg.base = base;
    const uint32_t klim = min(kend, g.Vne - 1u);
    if (lane < EPL)
        heads[lane] = 0u;
    __syncwarp();
    for (uint32_t j = k0 + 1u + (uint32_t)lane; j <= klim; j += 32u) {
        const uint64_t p = g.dst_off[j] - base;
        if (p < TILE_E) {
            atomicOr(&heads[(uint32_t)p >> 5], 1u << (uint32_t)(p & 31u));
            fill(j - k0, j);
        }
    }
    if (lane == 0)
        fill(0u, k0);
    __syncwarp();
    // prefix popcount of the EPL head words
    const uint32_t hw_own = (lane < EPL) ? heads[lane] : 0u;
    uint32_t incl = __popc(hw_own);
#pragma unroll
    for (int d = 1; d < EPL; d <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, incl, d);
        if (lane >= d)
            incl += y;
    }
    const uint32_t total = __shfl_sync(FULL, incl, EPL - 1);
    const uint32_t pos0 = (uint32_t)lane * EPL;
    const uint32_t wi = pos0 >> 5, sh = pos0 & 31u;
    const uint32_t word = heads[wi];
    const uint32_t excl_w = __shfl_sync(FULL, incl - __popc(hw_own), (int)wi);
    tg.k0 = k0;
    tg.k0_fresh = g.dst_off[k0] == base;
    const uint32_t k_last = k0 + total;
    tg.tail_cont = !last_tile && (kend == k_last);
    tg.ndst = total + 1u;
    tg.before = excl_w + __popc(word & ((1u << sh) - 1u));
    tg.nib_inner = (word >> sh) & ((EPL >= 32) ? FULL : ((1u << EPL) - 1u));
    tg.nib = tg.nib_inner | ((lane == 0 && tg.k0_fresh) ? 1u : 0u);
    __syncwarp();
}

// Destination ranks inside a tile, from the destination-start bitmap (bit p
// of g.dst_start: in-edge p is the first in-edge of its destination): position
// p belongs to compressed destination k0 + (number of starts in [1, p]).  Lane
// l < EPL loads word l of the tile and the words are prefix-counted with a
// shuffle scan: no loads of dst_off and no shared memory.  k0 / kend are the
// compressed destinations owning the tile's first edge and the next tile's
// first edge; base is a multiple of 32*EPL.
template <int EPL>
__device__ __forceinline__ void tile_geometry_bits(const DevGraph& g, uint64_t base, bool last_tile, uint32_t k0,
                                                   uint32_t kend, int lane, TileGeo<EPL>& tg)
{
    tg.base = base;
    uint32_t hw_own = (lane < EPL) ? g.dst_start[(base >> 5) + (uint32_t)lane] : 0u;
    const uint32_t w0 = __shfl_sync(FULL, hw_own, 0);
    tg.k0_fresh = (w0 & 1u) != 0u; /* k0 starts exactly at the tile start */
    if (lane == 0)
        hw_own &= ~1u; /* heads count the starts at positions [1, 32*EPL) */
    uint32_t incl = __popc(hw_own);
#pragma unroll
    for (int d = 1; d < EPL; d <<= 1) {
        const uint32_t y = __shfl_up_sync(FULL, incl, d);
        if (lane >= d)
            incl += y;
    }
    const uint32_t total = __shfl_sync(FULL, incl, EPL - 1);
    const uint32_t pos0 = (uint32_t)lane * EPL;
    const uint32_t wi = pos0 >> 5, sh = pos0 & 31u;
    const uint32_t word = __shfl_sync(FULL, hw_own, (int)wi);
    const uint32_t excl_w = __shfl_sync(FULL, incl - __popc(hw_own), (int)wi);
    tg.k0 = k0;
    const uint32_t k_last = k0 + total;
    tg.tail_cont = !last_tile && (kend == k_last);
    tg.ndst = total + 1u;
    tg.before = excl_w + __popc(word & ((1u << sh) - 1u));
    tg.nib_inner = (word >> sh) & ((EPL >= 32) ? FULL : ((1u << EPL) - 1u));
    tg.nib = tg.nib_inner | ((lane == 0 && tg.k0_fresh) ? 1u : 0u);
}

template <int EPL>
__device__ __forceinline__ uint32_t pos_dst(const TileGeo<EPL>& tg, int i)
{
    return tg.k0 + tg.before + __popc(tg.nib_inner & ((2u << i) - 1u));
}

// compressed destination owning in-edge position pos, from the destination-start
// bitmap and the 128-edge tile index: the owner of the index tile's first edge
// plus the destination starts after it
__device__ __forceinline__ uint32_t dst_of_pos(const uint32_t* dst_start, const uint32_t* tile_dst0, uint32_t pos)
{
    const uint32_t t = pos >> 7, w0 = t << 2, wp = pos >> 5;
    uint32_t n = 0;
    for (uint32_t w = w0; w < wp; ++w)
        n += __popc(dst_start[w]);
    n += __popc(dst_start[wp] & ((pos & 31u) == 31u ? FULL : ((2u << (pos & 31u)) - 1u)));
    return tile_dst0[t] + n - (dst_start[w0] & 1u); /* a start at the index tile's first edge is the owner's */
}

__device__ __forceinline__ uint32_t dst_of_pos(const DevGraph& g, uint32_t pos)
{
    return dst_of_pos(g.dst_start, g.tile_dst0, pos);
}

// (value, compensation) pair for the FP32 compensated PageRank sums
struct F2 {
    float s, c;
};
// warp shuffle-up of every value type the segmented reduction carries
template <class T>
__device__ __forceinline__ T shfl_up(T x, int d)
{
    return __shfl_up_sync(FULL, x, d);
}
template <>
__device__ __forceinline__ F2 shfl_up<F2>(F2 x, int d)
{
    return F2{__shfl_up_sync(FULL, x.s, d), __shfl_up_sync(FULL, x.c, d)};
}
// Knuth two-sum of the leading parts, compensations added
struct AddF2 {
    __device__ __forceinline__ F2 operator()(F2 a, F2 b) const
    {
        const float t = __fadd_rn(a.s, b.s);
        const float bp = __fsub_rn(t, a.s);
        const float err = __fadd_rn(__fsub_rn(a.s, __fsub_rn(t, bp)), __fsub_rn(b.s, bp));
        return F2{t, __fadd_rn(__fadd_rn(a.c, b.c), err)};
    }
};

enum : int { EMIT_COMPLETE = 0, EMIT_HEAD = 1, EMIT_TAIL = 2 };

// Segmented reduction of the tile's 32*EPL values; calls emit(k, value, kind)
// once per destination segment, on the lane holding the segment's last
// position.  kind: EMIT_COMPLETE (all in-edges of k are in this tile),
// EMIT_HEAD (k began in an earlier tile and ends here), EMIT_TAIL (k
// continues into the next tile).
template <int EPL, class T, class Op, class Emit>
__device__ __forceinline__ void seg_reduce(const T (&v)[EPL], const TileGeo<EPL>& tg, int lane, Op op, Emit emit)
{
    const uint32_t nib = tg.nib;
    T run = v[0];
    T first = v[0];
    int first_end = -1;
    int last_start = 0;
#pragma unroll
    for (int i = 1; i < EPL; ++i) {
        if ((nib >> i) & 1u) {
            if (first_end < 0) {
                first = run;
                first_end = i - 1;
                if (nib & 1u) {
                    const uint32_t k = pos_dst(tg, i - 1);
                    emit(k, run, (k == tg.k0 && !tg.k0_fresh) ? EMIT_HEAD : EMIT_COMPLETE);
                }
            } else {
                emit(pos_dst(tg, i - 1), run, EMIT_COMPLETE);
            }
            run = v[i];
            last_start = i;
        } else {
            run = op(run, v[i]);
        }
    }
    // inclusive segmented scan of the lanes' last runs
    bool f = (last_start > 0) || (nib & 1u);
    T s = run;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const T y = shfl_up(s, d);
        const bool gflag = __shfl_up_sync(FULL, f, d);
        if (lane >= d) {
            if (!f)
                s = op(y, s);
            f = f || gflag;
        }
    }
    const T sp = shfl_up(s, 1);
    const uint32_t next_fresh = __shfl_down_sync(FULL, nib & 1u, 1);
    if (first_end >= 0 && !(nib & 1u)) {
        const uint32_t k = pos_dst(tg, first_end);
        const T total = lane > 0 ? op(sp, first) : first;
        emit(k, total, (k == tg.k0 && !tg.k0_fresh) ? EMIT_HEAD : EMIT_COMPLETE);
    }
    if (lane == 31 || next_fresh) {
        const uint32_t k = pos_dst(tg, EPL - 1);
        int kind = EMIT_COMPLETE;
        if (lane == 31 && tg.tail_cont)
            kind = EMIT_TAIL;
        else if (k == tg.k0 && !tg.k0_fresh)
            kind = EMIT_HEAD;
        emit(k, s, kind);
    }
}

struct MinU32 {
    __device__ __forceinline__ uint32_t operator()(uint32_t a, uint32_t b) const { return min(a, b); }
};
struct MinU64 {
    __device__ __forceinline__ unsigned long long operator()(unsigned long long a, unsigned long long b) const
    {
        return a < b ? a : b;
    }
};
struct AddF64 {
    __device__ __forceinline__ double operator()(double a, double b) const { return __dadd_rn(a, b); }
};

}  // namespace wedge
