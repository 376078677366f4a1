/* include/gr.h compiled as C (not C++): the header is usable from C, and this
 * program prints the size and field offsets of the records that cross the ABI,
 * which tests/test_abi_consumers.py compares with the Python binding's ctypes
 * structures. No GPU work: it only calls gr_version and gr_status_string. */
#include <stddef.h>
#include <stdio.h>

#include "gr.h"

#define REC(T) printf("%s size %zu\n", #T, sizeof(T))
#define FIELD(T, f) printf("%s.%s %zu\n", #T, #f, offsetof(T, f))

int main(void) {
    REC(gr_ray); REC(gr_hit);
    REC(gr_opts); FIELD(gr_opts, flags);
    REC(gr_trace_tuning); REC(gr_tuning_result); FIELD(gr_tuning_result, ms);
    REC(gr_material); FIELD(gr_material, ior); FIELD(gr_material, color_map); FIELD(gr_material, uv_offset);
    FIELD(gr_material, specular);
    REC(gr_mesh); FIELD(gr_mesh, texcoords);
    REC(gr_camera); FIELD(gr_camera, fov_deg);
    REC(gr_environment); FIELD(gr_environment, map); FIELD(gr_environment, to_world);
    REC(gr_render_opts); FIELD(gr_render_opts, seed); FIELD(gr_render_opts, wave_paths);
    REC(gr_render_stats); FIELD(gr_render_stats, device_errors);
    REC(gr_server_opts); FIELD(gr_server_opts, policy); FIELD(gr_server_opts, age_cap_s);
    FIELD(gr_server_opts, max_wait_s);
    REC(gr_job_stats); FIELD(gr_job_stats, status); FIELD(gr_job_stats, waves); FIELD(gr_job_stats, last_wave);
    REC(gr_server_stats); FIELD(gr_server_stats, busy_s); FIELD(gr_server_stats, rejected);
    printf("version %d\n", gr_version());
    printf("status8 %s\n", gr_status_string(GR_ERR_BUSY));
    return 0;
}
