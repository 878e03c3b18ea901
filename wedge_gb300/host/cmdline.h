/*
 * Command line of the GPU `wedge` program.  Same options, defaults and exit
 * codes as the reference's command line (include/cmdline.h:26-57,
 * source/cmdline.c:65-529); -n and -u are accepted for compatibility and
 * ignored (there is one GPU and no NUMA placement).  Extra long options select
 * the GPU-only features.
 */
#ifndef WEDGE_HOST_CMDLINE_H
#define WEDGE_HOST_CMDLINE_H

#include <stdint.h>

#define CMDLINE_DEFAULT_NUM_THREADS 0
#define CMDLINE_DEFAULT_NUM_ITERATIONS 1
#define CMDLINE_DEFAULT_ROOT_VERTEX 0
#define CMDLINE_DEFAULT_FRONTIER_THRESHOLD_PCT 20

typedef struct cmdline_opts {
    char graph_input_filename[1024]; /* -i, required */
    char* graph_application_output_filename; /* -o */
    char application[64];            /* -a, required */
    uint32_t num_iterations;         /* -N */
    uint32_t num_threads;            /* -n (ignored) */
    uint64_t root_vertex;            /* -r */
    uint64_t frontier_threshold_pct; /* -t */
    int sched;                       /* --sched=plain|dense|wedge|filtered|learned */
    int precision;                   /* --prec=fp64|fp32c */
    double damping;                  /* --damping=<d>, 0 = reference value */
    int weights_f64;                 /* --weights=u64|f64 */
    int use_graph;                   /* --graph: CUDA-graph traversal loop */
    int timing;                      /* --timing: per-phase CUDA events */
    int iteration_stats;             /* --iteration-stats: the ITERATION_STATS CSV on stderr */
    char* scheduler_file;            /* --scheduler=<file>: network for --sched=learned */
} cmdline_opts_t;

void cmdline_parse_options_or_die(int argc, char* argv[]);
const cmdline_opts_t* cmdline_get_current_settings(void);

#endif
