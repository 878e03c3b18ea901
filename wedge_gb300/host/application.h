/*
 * Application registry of the GPU `wedge` program: the reference's names and
 * aliases (source/application.c:49-68), its per-application flags
 * (application.c:117-184) and its per-vertex output formats
 * (execution_{bfs,cc,pr,sssp}.c get_vertex_prop_string).
 */
#ifndef WEDGE_HOST_APPLICATION_H
#define WEDGE_HOST_APPLICATION_H

#include <stdbool.h>
#include <stddef.h>
#include <stdint.h>

typedef struct application_info {
    int app;                      /* enum wedge_app */
    const char* name;             /* canonical name (application.c:61-68) */
    bool has_special_output_stat; /* PageRank Sum */
    bool needs_wedge_frontier;
    bool uses_edge_weights;
} application_info_t;

/* application_select (application.c:197-205): case-insensitive exact match */
bool application_select(const char* appname, application_info_t* out);

/* one line of the -o output for vertex v, given the raw 64-bit property word
 * and (PageRank) the vertex's out-degree and the vertex count */
void application_prop_string(const application_info_t* app, uint64_t prop, uint64_t outdeg, uint64_t num_vertices,
                             int sssp_f64, char* buf, size_t size);

#endif
