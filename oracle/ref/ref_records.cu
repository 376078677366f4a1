// Host library built by build_ref.sh (here, where the reference sources are):
// builds reference scene records with the reference's own host code, so that
// tests can pin the byte-level restatement of those records in ref_gpu.py —
// which is what lays them out on the GPU machine, where this x86 library cannot run.
//   ref_camera_record: Camera() then Camera::setup(toWorld, fov, w, h, free =
//     false) (camera.h:10-38, transform.cpp), as the reference's loader calls it
//     for a perspective sensor (mitsubaloader.cpp:274-280);
//   ref_env_record: EnvironmentLight::setup(radiance) (environment.cpp:40-46)
//     with its world centre, viewed as EnvironmentLightView (environment.cpp:3-9).
// Records are copied out byte for byte; pointer fields hold host addresses.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <device_launch_parameters.h>
#include "renderer/pathtracer_kernel.h"

extern "C" {

int ref_camera_record(const float* to_world, float fov_deg, uint32_t width, uint32_t height, uint8_t* out,
                      uint32_t out_size) {
    if (out_size != sizeof(Camera)) return -1;
    float m[4][4];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) m[r][c] = to_world[4 * r + c];
    Camera cam;
    std::memset(static_cast<void*>(&cam), 0, sizeof(Camera));
    new (&cam) Camera();
    cam.setup(Transform(m), fov_deg, width, height, false);
    std::memcpy(out, &cam, sizeof(Camera));
    return 0;
}

int ref_env_record(int has, const float* radiance, const float* world_center, uint8_t* out, uint32_t out_size) {
    if (out_size != sizeof(EnvironmentLightView)) return -1;
    static EnvironmentLight env;  // keeps the buffer the view points at alive
    env = EnvironmentLight();
    if (has) env.setup(Spectrum(radiance[0], radiance[1], radiance[2]));
    else env.m_width = env.m_height = 0;
    env.m_world_center = make_float3(world_center[0], world_center[1], world_center[2]);
    EnvironmentLightView v = env.view();
    std::memset(out, 0, out_size);
    std::memcpy(out, &v, sizeof(v));
    return 0;
}

}  // extern "C"
