/* A C99 consumer of the C ABI: include/gbfv.h compiles as C, libgbfv.so
 * links, and the entry points that need no device run (default
 * parameters, restart file text and names, the footprint estimate). */
#include <stdio.h>
#include <string.h>

#include "gbfv.h"

int main(void)
{
    gbfv_params p;
    gbfv_default_params(&p);
    if (p.newton_max_iterations != 20 || p.local_linearizer != GBFV_LIN_AD) return 1;

    gbfv_restart_info info;
    memset(&info, 0, sizeof info);
    info.num_cpus = 1;
    info.num_edges = 7;
    info.num_vertices = 6;
    info.time = 250.0;
    info.time_step_index = 1;
    const double pv[4] = {1e5, 0.5, 1.25e5, 0.25};
    size_t len = 0;
    if (gbfv_format_restart(&info, 2, 2, pv, NULL, NULL, 0, &len) != GBFV_OK) return 2;
    char text[1024];
    if (len > sizeof text || gbfv_format_restart(&info, 2, 2, pv, NULL, text, sizeof text, &len) != GBFV_OK)
        return 3;
    double back[4];
    gbfv_restart_info out;
    if (gbfv_parse_restart(text, len, &info, 2, 2, back, NULL, &out) != GBFV_OK) return 4;
    if (memcmp(back, pv, sizeof pv) != 0 || out.time != 250.0) return 5;

    char name[256];
    if (gbfv_restart_file_name("out", "lens", 250.0, 0, name, sizeof name) != GBFV_OK) return 6;
    if (strcmp(name, "out/lens_time=250_rank=0.ers") != 0) return 7;
    if (gbfv_footprint_bytes(200000, 3, 3) <= 0) return 8;

    printf("abi ok %zu\n", len);
    return 0;
}
