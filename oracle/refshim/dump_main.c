/*
 * Test infrastructure only: a replacement `main` for the reference build in
 * `oracle/_ref/`.  It follows the reference's own program flow
 * (source/main.c:33-110: application_select -> graph_data_read_from_file ->
 * graph_data_initialize_data_structures -> parameters -> spindleThreadsSpawn
 * (application_execute)) and then, instead of the 5-significant-digit text
 * output, dumps the raw 64-bit vertex properties (and, for PageRank, the
 * out-degrees) so the oracle can be compared bit-for-bit.
 *
 * usage: wedge_ref <graph> <app> <threads> <iterations> <root> <threshold_pct> <out.bin>
 * stdout: one JSON line with the run statistics (source/main.c:153-170).
 * out.bin: uint64 V, then V uint64 props, then (PR only) V uint64 outdegree words.
 */
#include <stdbool.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include "application.h"
#include "execution.h"
#include "graphdata.h"

#include <spindle.h>

extern uint32_t shim_default_threads;

int main(int argc, char** argv)
{
    if (argc != 8) {
        fprintf(stderr, "usage: %s graph app threads iterations root threshold out.bin\n", argv[0]);
        return 2;
    }
    const char* path = argv[1];
    const char* app = argv[2];
    const uint32_t threads = (uint32_t)strtoul(argv[3], NULL, 10);
    const uint64_t iters = strtoull(argv[4], NULL, 10);
    const uint64_t root = strtoull(argv[5], NULL, 10);
    const uint64_t thr = strtoull(argv[6], NULL, 10);
    uint32_t nodes[1] = {0};
    shim_default_threads = threads;

    if (!application_select(app)) {
        fprintf(stderr, "bad app %s\n", app);
        return 3;
    }
    if (!graph_data_read_from_file(path, 1, nodes))
        return 4;
    /* The reference's main sets these after graph_data_initialize_data_structures
     * (main.c:75-79), whose execution_initialize_* already seeds the root from
     * graph_param_root_vertex -- still 0 then, so `-r` does not move the BFS/SSSP
     * root there.  Setting them first gives `-r` its documented meaning. */
    graph_param_num_static_iterations = iters;
    graph_param_root_vertex = root < graph_num_vertices ? root : 0;
    graph_param_frontier_threshold_pct = thr;
    graph_data_initialize_data_structures(threads, 1, nodes);

    SSpindleTaskSpec spec;
    spec.func = &application_execute;
    spec.arg = NULL;
    spec.numaNode = 0;
    spec.numThreads = threads;
    spec.smtPolicy = SpindleSMTPolicyPreferPhysical;
    spindleThreadsSpawn(&spec, 1, true);

    FILE* f = fopen(argv[7], "wb");
    if (!f)
        return 5;
    fwrite(&graph_num_vertices, 8, 1, f);
    fwrite(graph_vertex_props, 8, graph_num_vertices, f);
    if (execution_has_special_output_stat)
        fwrite(graph_vertex_outdegrees, 8, graph_num_vertices, f);
    fclose(f);

    const double pull = total_processing_time_nowedge + total_processing_time_wedge;
    printf("{\"vertices\": %llu, \"edges\": %llu, \"edge_vectors\": %llu, \"iterations\": %llu, "
           "\"wedge_iterations\": %llu, \"running_ms\": %.6f, \"pull_ms\": %.6f, \"wedge_ms\": %.6f}\n",
           (unsigned long long)graph_num_vertices, (unsigned long long)graph_num_edges,
           (unsigned long long)graph_num_edge_vectors, (unsigned long long)total_iterations_executed,
           (unsigned long long)total_wedge_iterations_executed, pull + total_activation_time, pull,
           total_activation_time);
    return 0;
}
