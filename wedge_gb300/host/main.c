/*
 * GPU `wedge` program: the reference's program flow (source/main.c:33-185)
 * with the edge-pull engine on the GPU behind the C ABI of wedge_cuda.h:
 *   parse -> application_select -> wedge_cuda_load_graph -> wedge_cuda_run
 *   -> optional -o output -> EXECUTION STATISTICS block.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "application.h"
#include "cmdline.h"
#include "wedge_cuda.h"

static double now_ms(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec * 1000.0 + (double)ts.tv_nsec / 1e6;
}

int main(int argc, char* argv[])
{
    cmdline_parse_options_or_die(argc, argv);
    const cmdline_opts_t* o = cmdline_get_current_settings();

    printf("Frontier:    precision set to 32 in-edges/bit\n");
    printf("Frontier:    threshold set to %llu%%\n", (unsigned long long)o->frontier_threshold_pct);

    application_info_t app;
    if (!application_select(o->application, &app)) {
        printf("Application: ERROR: unable to run \"%s\"\n", o->application);
        return __LINE__;
    }
    printf("Application: %s on the GPU\n", app.name);

    printf("Graph:       reading \"%s\"\n", o->graph_input_filename);
    const double t0 = now_ms();
    wedge_graph_t* g = NULL;
    const int wk = app.uses_edge_weights ? (o->weights_f64 ? WEDGE_WEIGHTS_F64 : WEDGE_WEIGHTS_U64) : WEDGE_WEIGHTS_NONE;
    int rc = wedge_cuda_load_graph_ex(o->graph_input_filename, app.app, wk, &g);
    if (rc != WEDGE_OK) {
        printf("Graph:       ERROR: %s\n", wedge_cuda_status_string(rc));
        return __LINE__;
    }
    const uint64_t V = wedge_cuda_num_vertices(g), E = wedge_cuda_num_edges(g);
    printf("Graph:       contains %llu vertices and %llu edges\n", (unsigned long long)V, (unsigned long long)E);
    printf("Graph:       loading completed in %.2lf msec\n", now_ms() - t0);

    uint64_t root = o->root_vertex;
    if (root >= V) {
        printf("Application: WARNING: root vertex %llu is out of range, using %d instead\n", (unsigned long long)root,
               CMDLINE_DEFAULT_ROOT_VERTEX);
        root = CMDLINE_DEFAULT_ROOT_VERTEX;
    }
    wedge_params_t p;
    memset(&p, 0, sizeof(p));
    p.root = root;
    p.threshold_pct = (uint32_t)o->frontier_threshold_pct;
    p.num_iterations = o->num_iterations;
    p.damping = o->damping;
    p.precision = o->precision;
    p.sched = o->sched;
    /* the ITERATION_STATS rows carry measured pull and Wedge times (execution_bfs.c:227-232) */
    p.flags = (o->use_graph ? WEDGE_FLAG_GRAPH : 0u) | ((o->timing || o->iteration_stats) ? WEDGE_FLAG_TIMING : 0u);
    if (o->sched == WEDGE_SCHED_LEARNED) {
        if (!o->scheduler_file) {
            printf("Application: ERROR: --sched=learned needs --scheduler=<file>\n");
            wedge_cuda_free(g);
            return __LINE__;
        }
        float blob[WEDGE_SCHED_BLOB];
        FILE* nf = fopen(o->scheduler_file, "rb");
        const size_t got = nf ? fread(blob, sizeof(float), WEDGE_SCHED_BLOB, nf) : 0;
        if (nf)
            fclose(nf);
        if (got != WEDGE_SCHED_BLOB || wedge_cuda_set_scheduler(g, blob, WEDGE_SCHED_BLOB) != WEDGE_OK) {
            printf("Application: ERROR: unable to load the scheduler network \"%s\"\n", o->scheduler_file);
            wedge_cuda_free(g);
            return __LINE__;
        }
    }
    printf("Application: starting execution\n");
    wedge_stats_t st;
    rc = wedge_cuda_run(g, app.app, &p, &st);
    if (rc != WEDGE_OK && rc != WEDGE_ERR_NOT_CONVERGED) {
        printf("Application: ERROR: %s\n", wedge_cuda_status_string(rc));
        wedge_cuda_free(g);
        return __LINE__;
    }
    if (rc == WEDGE_ERR_NOT_CONVERGED)
        printf("Application: WARNING: %s\n", wedge_cuda_status_string(rc));
    printf("Application: completed execution\n");

    if (o->iteration_stats && app.app != WEDGE_APP_PR) {
        /* EXPERIMENT_ITERATION_STATS rows (execution_bfs.c:227-232), one per iteration */
        uint64_t n = 0;
        if (wedge_cuda_iteration_log(g, NULL, 0, &n) == WEDGE_OK && n) {
            wedge_iteration_record_t* recs = (wedge_iteration_record_t*)malloc(n * sizeof(*recs));
            if (recs && wedge_cuda_iteration_log(g, recs, n, &n) == WEDGE_OK)
                for (uint64_t i = 0; i < n; ++i)
                    fprintf(stderr, "%llu,%s,%lf,%lf\n", (unsigned long long)recs[i].active_edges,
                            recs[i].used_wedge ? "true" : "false", recs[i].pull_ms, recs[i].wedge_ms);
            free(recs);
        }
    }

    if (o->graph_application_output_filename) {
        /* source/main.c:112-150, formatted on the GPU where the format allows */
        const double t1 = now_ms();
        printf("Application: writing output to \"%s\"\n", o->graph_application_output_filename);
        int on_gpu = 0;
        double fmt_ms = 0.0;
        rc = wedge_cuda_write_output(g, o->graph_application_output_filename, &on_gpu, &fmt_ms);
        if (rc == WEDGE_ERR_IO)
            printf("Application: ERROR: unable to write to \"%s\"\n", o->graph_application_output_filename);
        else if (rc != WEDGE_OK)
            printf("Application: ERROR: %s\n", wedge_cuda_status_string(rc));
        else
            printf("Application: writing completed in %.2lf msec (formatting %.2lf msec on the %s)\n", now_ms() - t1,
                   fmt_ms, on_gpu ? "GPU" : "host");
    }

    /* source/main.c:153-182 */
    const double pull = st.pull_ms_dense + st.pull_ms_wedge;
    printf("\n--------------- EXECUTION STATISTICS ---------------\n");
    printf("%-28s = %.2lf msec\n", "Running Time", st.running_ms);
    printf("%-28s = %.4lf Bedges/sec\n", "Effective Throughput",
           (double)E * (double)st.iterations / st.running_ms / 1000000.0);
    printf("%-28s = %.4lf\n", "GTEPS (|E| per traversal)", (double)E / st.running_ms / 1000000.0);
    printf("----------------------------------------------------\n");
    printf("%-28s = %.2lf msec\n", "Pull Time", pull);
    printf("%-28s = %.2lf msec\n", "Frontier Pull Time", st.pull_ms_wedge);
    printf("%-28s = %.2lf msec\n", "No Frontier Pull Time", st.pull_ms_dense);
    printf("%-28s = %.2lf msec\n", "Wedge Time", st.wedge_ms);
    printf("----------------------------------------------------\n");
    printf("%-28s = %llu\n", "Total Iterations", (unsigned long long)st.iterations);
    printf("%-28s = %llu\n", "Iterations with Wedge", (unsigned long long)st.wedge_iterations);
    printf("%-28s = %llu\n", "Iterations without Wedge", (unsigned long long)(st.iterations - st.wedge_iterations));
    printf("%-28s = %llu\n", "In-edges Scanned", (unsigned long long)st.edges_scanned);
    printf("----------------------------------------------------\n");
    if (app.has_special_output_stat) {
        printf("%-28s = %.8lf\n", "PageRank Sum", st.pr_sum);
        printf("----------------------------------------------------\n");
    }
    printf("\n");
    wedge_cuda_free(g);
    return 0;
}
