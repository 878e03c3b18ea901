/*
 * wedge-gen: writes the seeded synthetic graphs in the reference's binary edge
 * list format (README.md:42-50; read by graph_data_read_from_file,
 * graphdata.c:946-1133): a header of two uint64 words (vertices, edges), then
 * one (src, dst) pair of uint64 words per edge, or (src, dst, weight) for
 * weighted graphs, grouped by destination in ascending order.
 *
 *   wedge-gen rmat <scale> <edge-factor> <seed> [--sym] [--weights=u64|f64] -o <file>
 *   wedge-gen grid <side> <long-range-fraction> <seed> [--weights=u64|f64] -o <file>
 *
 * The edge lists come from the engine's device generators (R-MAT with
 * a/b/c = 0.57/0.19/0.19 from a counter-based splitmix64 draw; the 4-neighbour
 * grid in both directions plus floor(fraction * 4*side*(side-1)) random pairs),
 * sorted by (dst, src).  Weights are the multiplicative hash of (src, dst):
 * h = ((src << 32) | dst) * 0x9E3779B97F4A7C15 mod 2^64, uint64 weight
 * 1 + (((h >> 32) * 255) >> 32), FP64 weight h * 2^-64 -- the same words the
 * engine computes when it generates a weighted graph itself.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "wedge_cuda.h"

static int usage(void)
{
    printf("usage: wedge-gen rmat <scale> <edge-factor> <seed> [--sym] [--weights=u64|f64] -o <file>\n"
           "       wedge-gen grid <side> <long-range-fraction> <seed> [--weights=u64|f64] -o <file>\n");
    return 1;
}

static uint64_t weight_word(uint32_t s, uint32_t d, int f64)
{
    const uint64_t h = (((uint64_t)s << 32) | d) * 0x9E3779B97F4A7C15ull;
    if (f64) {
        const double x = (double)h * 0x1p-64; /* the conversion rounds to nearest; the scaling is exact */
        uint64_t bits;
        memcpy(&bits, &x, sizeof(bits));
        return bits;
    }
    return 1ull + (((h >> 32) * 255ull) >> 32);
}

static int write_edges(const char* path, uint64_t V, uint64_t E, const uint32_t* src, const uint32_t* dst,
                       int weights, int f64)
{
    FILE* f = fopen(path, "wb");
    if (!f)
        return 0;
    const uint64_t hdr[2] = {V, E};
    int ok = fwrite(hdr, 8, 2, f) == 2;
    const uint64_t tup = weights ? 3u : 2u;
    static uint64_t buf[3 * 4096];
    uint64_t n = 0;
    for (uint64_t e = 0; e < E && ok; ++e) {
        buf[n++] = src[e];
        buf[n++] = dst[e];
        if (weights)
            buf[n++] = weight_word(src[e], dst[e], f64);
        if (n == tup * 4096u) {
            ok = fwrite(buf, 8, n, f) == n;
            n = 0;
        }
    }
    if (n && ok)
        ok = fwrite(buf, 8, n, f) == n;
    return (fclose(f) == 0) && ok;
}

int main(int argc, char* argv[])
{
    if (argc < 5)
        return usage();
    const int rmat = !strcmp(argv[1], "rmat");
    if (!rmat && strcmp(argv[1], "grid"))
        return usage();
    const char* out = NULL;
    int sym = 0, weights = 0, f64 = 0;
    for (int i = 5; i < argc; ++i) {
        if (rmat && !strcmp(argv[i], "--sym"))
            sym = 1;
        else if (!strcmp(argv[i], "--weights=u64"))
            weights = 1;
        else if (!strcmp(argv[i], "--weights=f64"))
            weights = f64 = 1;
        else if (!strcmp(argv[i], "-o") && i + 1 < argc)
            out = argv[++i];
        else
            return usage();
    }
    if (!out)
        return usage();
    const uint64_t seed = strtoull(argv[4], NULL, 10);
    const uint32_t a = (uint32_t)strtoul(argv[2], NULL, 10);
    const uint32_t ef = rmat ? (uint32_t)strtoul(argv[3], NULL, 10) : 0u;
    const double frac = rmat ? 0.0 : strtod(argv[3], NULL);
    uint64_t V = 0, E = 0;
    int rc = rmat ? wedge_cuda_rmat_edge_list(a, ef, 0.57, 0.19, 0.19, seed, sym, &V, &E, NULL, NULL, 0)
                  : wedge_cuda_grid_edge_list(a, frac, seed, &V, &E, NULL, NULL, 0);
    uint32_t* src = NULL;
    uint32_t* dst = NULL;
    if (rc == WEDGE_OK) {
        src = (uint32_t*)malloc(4 * (E ? E : 1));
        dst = (uint32_t*)malloc(4 * (E ? E : 1));
        if (!src || !dst)
            rc = WEDGE_ERR_OOM;
        else
            rc = rmat ? wedge_cuda_rmat_edge_list(a, ef, 0.57, 0.19, 0.19, seed, sym, &V, &E, src, dst, E)
                      : wedge_cuda_grid_edge_list(a, frac, seed, &V, &E, src, dst, E);
    }
    if (rc != WEDGE_OK) {
        printf("wedge-gen: %s\n", wedge_cuda_status_string(rc));
        free(src);
        free(dst);
        return 2;
    }
    const int ok = write_edges(out, V, E, src, dst, weights, f64);
    free(src);
    free(dst);
    if (!ok) {
        printf("wedge-gen: write error on \"%s\"\n", out);
        return 3;
    }
    printf("wedge-gen: wrote %llu vertices, %llu edges to \"%s\"\n", (unsigned long long)V, (unsigned long long)E, out);
    return 0;
}
