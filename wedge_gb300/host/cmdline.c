/*
 * Command-line parsing for the GPU `wedge` program.  Option letters, required
 * options, defaults and the exit codes of each error (1 unknown option,
 * 2 invalid value, 3 missing value, 4 extraneous value, 5 missing required
 * option) follow source/cmdline.c:128-179 so scripts written for the reference
 * keep working.
 */
#include "cmdline.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "wedge_cuda.h"

static cmdline_opts_t opts;

static void usage_and_exit(const char* argv0)
{
    printf("Usage: %s [options] -a application-name -i input-graph\n", argv0);
    printf("       %s -h\n       %s -V\n\n", argv0, argv0);
    printf("Required:\n");
    printf("  -a application-name   bfs | cc | pr | sssp (and the reference's long names)\n");
    printf("  -i input-graph        Wedge binary edge list, grouped by ascending destination\n\n");
    printf("Options:\n");
    printf("  -h                    Prints this information and exits.\n");
    printf("  -n num-threads        Accepted for compatibility; ignored on the GPU.\n");
    printf("  -N num-iterations     PageRank iterations. Defaults to %d.\n", CMDLINE_DEFAULT_NUM_ITERATIONS);
    printf("  -o output-file        Writes the final value of every vertex.\n");
    printf("  -r root-vertex        Root for BFS and SSSP. Defaults to %d.\n", CMDLINE_DEFAULT_ROOT_VERTEX);
    printf("  -t threshold          Active-edge percentage above which Wedge is skipped. Defaults to %d.\n",
           CMDLINE_DEFAULT_FRONTIER_THRESHOLD_PCT);
    printf("  -u node[,node...]     Accepted for compatibility; ignored on the GPU.\n");
    printf("  -V                    Prints version information and exits.\n");
    printf("  --sched=plain|dense|wedge|filtered|learned\n");
    printf("                              iteration strategy (default plain = fixed threshold)\n");
    printf("  --scheduler=<file>          network for --sched=learned (WEDGE_SCHED_BLOB floats)\n");
    printf("  --iteration-stats           per-iteration CSV on stderr: active edges, used Wedge, pull ms, Wedge ms\n");
    printf("  --prec=fp64|fp32c           PageRank arithmetic (default fp64)\n");
    printf("  --damping=<d>               PageRank damping (default 0.875, as the reference)\n");
    printf("  --weights=u64|f64           SSSP weight words (default u64, as the reference)\n");
    printf("  --graph                     run the traversal as one CUDA graph\n");
    printf("  --timing                    per-phase timing (Pull / Wedge times)\n");
    exit(0);
}

static void die(const char* argv0, int code, const char* fmt, const char* a, const char* b)
{
    printf("%s: ", argv0);
    printf(fmt, a, b);
    printf("\nTry `%s -h' for more information.\n", argv0);
    exit(code);
}

static int parse_u64(const char* s, uint64_t* out)
{
    char* end = NULL;
    if (!s || !*s)
        return 0;
    for (const char* p = s; *p; ++p)
        if (*p < '0' || *p > '9')
            return 0;
    *out = strtoull(s, &end, 10);
    return end && *end == '\0';
}

static int parse_long_option(const char* arg)
{
    if (strcmp(arg, "--graph") == 0) {
        opts.use_graph = 1;
        return 1;
    }
    if (strcmp(arg, "--timing") == 0) {
        opts.timing = 1;
        return 1;
    }
    if (strcmp(arg, "--iteration-stats") == 0) {
        opts.iteration_stats = 1;
        return 1;
    }
    if (strncmp(arg, "--scheduler=", 12) == 0) {
        if (!arg[12])
            return -1;
        opts.scheduler_file = (char*)arg + 12;
        return 1;
    }
    if (strncmp(arg, "--sched=", 8) == 0) {
        const char* v = arg + 8;
        if (!strcmp(v, "plain"))
            opts.sched = WEDGE_SCHED_PLAIN;
        else if (!strcmp(v, "dense"))
            opts.sched = WEDGE_SCHED_DENSE;
        else if (!strcmp(v, "wedge"))
            opts.sched = WEDGE_SCHED_WEDGE;
        else if (!strcmp(v, "filtered"))
            opts.sched = WEDGE_SCHED_FILTERED;
        else if (!strcmp(v, "learned"))
            opts.sched = WEDGE_SCHED_LEARNED;
        else
            return -1;
        return 1;
    }
    if (strncmp(arg, "--prec=", 7) == 0) {
        const char* v = arg + 7;
        if (!strcmp(v, "fp64"))
            opts.precision = WEDGE_PREC_FP64;
        else if (!strcmp(v, "fp32c"))
            opts.precision = WEDGE_PREC_FP32C;
        else
            return -1;
        return 1;
    }
    if (strncmp(arg, "--weights=", 10) == 0) {
        const char* v = arg + 10;
        if (!strcmp(v, "u64"))
            opts.weights_f64 = 0;
        else if (!strcmp(v, "f64"))
            opts.weights_f64 = 1;
        else
            return -1;
        return 1;
    }
    if (strncmp(arg, "--damping=", 10) == 0) {
        char* end = NULL;
        const double d = strtod(arg + 10, &end);
        if (!end || *end || !(d > 0.0 && d < 1.0))
            return -1;
        opts.damping = d;
        return 1;
    }
    return 0;
}

void cmdline_parse_options_or_die(int argc, char* argv[])
{
    memset(&opts, 0, sizeof(opts));
    opts.num_iterations = CMDLINE_DEFAULT_NUM_ITERATIONS;
    opts.num_threads = CMDLINE_DEFAULT_NUM_THREADS;
    opts.root_vertex = CMDLINE_DEFAULT_ROOT_VERTEX;
    opts.frontier_threshold_pct = CMDLINE_DEFAULT_FRONTIER_THRESHOLD_PCT;
    int have_a = 0, have_i = 0;
    for (int i = 1; i < argc; ++i) {
        const char* arg = argv[i];
        if (arg[0] == '-' && arg[1] == '-') {
            const int r = parse_long_option(arg);
            if (r == 1)
                continue;
            if (r < 0)
                die(argv[0], 2, "Invalid value in option `%s'.%s", arg, "");
            die(argv[0], 1, "Unrecognized option `%s'.%s", arg, "");
        }
        if (arg[0] != '-' || arg[1] == '\0' || arg[2] != '\0')
            die(argv[0], 1, "Unrecognized option `%s'.%s", arg, "");
        const char o = arg[1];
        if (o == 'h')
            usage_and_exit(argv[0]);
        if (o == 'V') {
            printf("Wedge (GB300 edge-pull engine, C ABI v%d)\n", wedge_cuda_abi_version());
            exit(0);
        }
        if (!strchr("ainNortu", o))
            die(argv[0], 1, "Unrecognized option `%s'.%s", arg, "");
        if (i + 1 >= argc)
            die(argv[0], 3, "Missing argument for option `%s'.%s", arg, "");
        const char* val = argv[++i];
        uint64_t u = 0;
        switch (o) {
        case 'a':
            if (strlen(val) >= sizeof(opts.application))
                die(argv[0], 2, "Invalid value `%s' for option `%s'.", val, arg);
            strcpy(opts.application, val);
            have_a = 1;
            break;
        case 'i':
            if (strlen(val) >= sizeof(opts.graph_input_filename))
                die(argv[0], 2, "Invalid value `%s' for option `%s'.", val, arg);
            strcpy(opts.graph_input_filename, val);
            have_i = 1;
            break;
        case 'o':
            opts.graph_application_output_filename = (char*)val;
            break;
        case 'n':
            if (!parse_u64(val, &u))
                die(argv[0], 2, "Invalid value `%s' for option `%s'.", val, arg);
            opts.num_threads = (uint32_t)u;
            break;
        case 'N':
            if (!parse_u64(val, &u) || u == 0 || u > 0xffffffffull)
                die(argv[0], 2, "Invalid value `%s' for option `%s'.", val, arg);
            opts.num_iterations = (uint32_t)u;
            break;
        case 'r':
            if (!parse_u64(val, &u))
                die(argv[0], 2, "Invalid value `%s' for option `%s'.", val, arg);
            opts.root_vertex = u;
            break;
        case 't':
            if (!parse_u64(val, &u) || u > 100)
                die(argv[0], 2, "Invalid value `%s' for option `%s'.", val, arg);
            opts.frontier_threshold_pct = u;
            break;
        case 'u':
            break;
        }
    }
    if (!have_a)
        die(argv[0], 5, "Missing required option `-%s'.%s", "a", "");
    if (!have_i)
        die(argv[0], 5, "Missing required option `-%s'.%s", "i", "");
}

const cmdline_opts_t* cmdline_get_current_settings(void) { return &opts; }
