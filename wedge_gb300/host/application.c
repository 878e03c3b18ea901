/*
 * Application registry and output formats of the GPU `wedge` program
 * (see application.h for the reference lines each part mirrors).
 */
#include "application.h"

#include <stdio.h>
#include <string.h>
#include <strings.h>

#include "wedge_cuda.h"

static const char* const names_bfs[] = {"bfs", "breadth_first_search", "breadthfirstsearch"};
static const char* const names_cc[] = {"cc", "connected_components", "connectedcomponents"};
static const char* const names_pr[] = {"pr", "pagerank"};
static const char* const names_sssp[] = {"sssp", "single_source_shortest_path", "singlesourceshortestpath"};

static bool match(const char* const* names, size_t n, const char* appname)
{
    for (size_t i = 0; i < n; ++i)
        if (strcasecmp(names[i], appname) == 0)
            return true;
    return false;
}

bool application_select(const char* appname, application_info_t* out)
{
    if (!appname || !out)
        return false;
    memset(out, 0, sizeof(*out));
    if (match(names_bfs, 3, appname)) {
        out->app = WEDGE_APP_BFS;
        out->name = "Breadth-First Search";
        out->needs_wedge_frontier = true;
    } else if (match(names_cc, 3, appname)) {
        out->app = WEDGE_APP_CC;
        out->name = "Connected Components";
        out->needs_wedge_frontier = true;
    } else if (match(names_pr, 2, appname)) {
        out->app = WEDGE_APP_PR;
        out->name = "PageRank";
        out->has_special_output_stat = true;
    } else if (match(names_sssp, 3, appname)) {
        out->app = WEDGE_APP_SSSP;
        out->name = "Single-Source Shortest Path";
        out->needs_wedge_frontier = true;
        out->uses_edge_weights = true;
    } else {
        return false;
    }
    return true;
}

void application_prop_string(const application_info_t* app, uint64_t prop, uint64_t outdeg, uint64_t num_vertices,
                             int sssp_f64, char* buf, size_t size)
{
    double d;
    memcpy(&d, &prop, sizeof(d));
    switch (app->app) {
    case WEDGE_APP_BFS: /* execution_bfs.c:69-73 */
        snprintf(buf, size, "%lld", (long long)prop);
        break;
    case WEDGE_APP_CC: /* execution_cc.c:47-51 */
        snprintf(buf, size, "%.0lf", d);
        break;
    case WEDGE_APP_PR: /* execution_pr.c:31-35 */
        snprintf(buf, size, "%.4le", d * (outdeg == 0 ? (double)num_vertices : (double)outdeg));
        break;
    default: /* execution_sssp.c:48-52 */
        if (sssp_f64)
            snprintf(buf, size, "%.17g", d);
        else
            snprintf(buf, size, "%lld", (long long)prop);
        break;
    }
}
