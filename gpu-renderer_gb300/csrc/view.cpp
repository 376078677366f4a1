// View operations on a scene: camera get / set, the interactive camera moves of
// the reference's viewer (zoom, translate, rotate, resize) and the 8-bit output
// step. Each camera change restarts the accumulation, as the reference's
// m_reset flag does at its next render (pathtracer.cu:172-213).
//
// The reference applies zoom / translate / rotate to its free-flying camera
// state (eye, direction, yaw, pitch; camera.h:40-62) and ignores them for a
// camera given by a to_world matrix. Here they act on the scene's to_world
// matrix itself, with the same meaning: zoom moves the eye along the view
// direction, translate moves it in the view plane (horizontal axis
// normalize(cross(dir, world up)), vertical axis normalize(cross(horizontal,
// dir))), rotate turns the view by yaw about the world up axis, then by pitch
// about the camera's horizontal axis.
#include <cmath>
#include <cstring>
#include <string>

#include "render.h"

namespace {

struct F3 {
    float x, y, z;
};

F3 add(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
F3 scale(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
F3 cross(F3 a, F3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
F3 normalize(F3 a) {
    const float l = std::sqrt(dot(a, a));
    return l > 0.0f ? scale(a, 1.0f / l) : a;
}

// to_world is row-major 4x4: column k of the upper 3x3 is camera axis k, column 3 the eye.
F3 column(const gr_camera& c, int k) { return {c.to_world[k], c.to_world[4 + k], c.to_world[8 + k]}; }
void set_column(gr_camera& c, int k, F3 v) {
    c.to_world[k] = v.x;
    c.to_world[4 + k] = v.y;
    c.to_world[8 + k] = v.z;
}

// Rodrigues rotation of v about the unit axis u by angle a.
F3 rotate_about(F3 v, F3 u, float a) {
    const float c = std::cos(a), s = std::sin(a);
    return add(add(scale(v, c), scale(cross(u, v), s)), scale(u, dot(u, v) * (1.0f - c)));
}

gr_status view_fail(gr_ctx* ctx, gr_status st, const std::string& what) {
    if (ctx) ctx->last_error = what;
    return st;
}

gr_status view_cuda(gr_ctx* ctx, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return GR_OK;
    return view_fail(ctx, GR_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

#define VIEW_CUDA(ctx, call)                                  \
    do {                                                      \
        const gr_status st__ = view_cuda(ctx, (call), #call); \
        if (st__ != GR_OK) return st__;                       \
    } while (0)

}  // namespace

extern "C" {

gr_status gr_scene_get_camera(const gr_scene* sc, gr_camera* out) {
    if (!sc || !out) return GR_ERR_INVALID;
    *out = sc->cam_rec;
    return GR_OK;
}

gr_status gr_scene_set_camera(gr_scene* sc, const gr_camera* cam) {
    if (!sc || !cam) return GR_ERR_INVALID;
    gr_ctx* ctx = sc->ctx;
    if (!gr::pixels_ok(cam->width, cam->height))
        return view_fail(ctx, GR_ERR_INVALID, "gr_scene_set_camera: bad resolution");
    if (!(cam->fov_deg > 0.0f && cam->fov_deg < 180.0f))
        return view_fail(ctx, GR_ERR_INVALID, "gr_scene_set_camera: field of view outside (0, 180) degrees");
    VIEW_CUDA(ctx, cudaSetDevice(ctx->device));
    VIEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const size_t npix = (size_t)cam->width * cam->height;
    VIEW_CUDA(ctx, sc->fb.ensure(24 * npix));
    VIEW_CUDA(ctx, sc->fb_count.ensure(4 * npix));
    sc->cam_rec = *cam;
    sc->cam = gr::make_camera(*cam);
    return gr_scene_reset(sc);
}

gr_status gr_scene_zoom(gr_scene* sc, float d) {
    if (!sc) return GR_ERR_INVALID;
    gr_camera c = sc->cam_rec;
    const F3 dir = normalize(column(c, 2));
    set_column(c, 3, add(column(c, 3), scale(dir, d)));
    return gr_scene_set_camera(sc, &c);
}

gr_status gr_scene_translate(gr_scene* sc, float x, float y) {
    if (!sc) return GR_ERR_INVALID;
    gr_camera c = sc->cam_rec;
    const F3 dir = normalize(column(c, 2));
    const F3 horizontal = normalize(cross(dir, F3{0.0f, 1.0f, 0.0f}));
    const F3 vertical = normalize(cross(horizontal, dir));
    set_column(c, 3, add(column(c, 3), add(scale(horizontal, x), scale(vertical, y))));
    return gr_scene_set_camera(sc, &c);
}

gr_status gr_scene_rotate(gr_scene* sc, float yaw, float pitch) {
    if (!sc) return GR_ERR_INVALID;
    gr_camera c = sc->cam_rec;
    const F3 up{0.0f, 1.0f, 0.0f};
    F3 axes[3] = {column(c, 0), column(c, 1), column(c, 2)};
    for (F3& a : axes) a = rotate_about(a, up, yaw);
    const F3 horizontal = normalize(cross(normalize(axes[2]), up));
    if (dot(horizontal, horizontal) > 0.0f)
        for (F3& a : axes) a = rotate_about(a, horizontal, pitch);
    for (int k = 0; k < 3; ++k) set_column(c, k, axes[k]);
    return gr_scene_set_camera(sc, &c);
}

gr_status gr_scene_resize(gr_scene* sc, uint32_t width, uint32_t height) {
    if (!sc) return GR_ERR_INVALID;
    gr_camera c = sc->cam_rec;
    c.width = width;
    c.height = height;
    return gr_scene_set_camera(sc, &c);
}

gr_status gr_scene_rgba8(gr_scene* sc, uint32_t* d_rgba, void* stream) {
    if (!sc || !d_rgba) return GR_ERR_INVALID;
    gr_ctx* ctx = sc->ctx;
    VIEW_CUDA(ctx, cudaSetDevice(ctx->device));
    cudaStream_t s = (cudaStream_t)stream;
    // the accumulation is written on the context stream
    cudaEvent_t ev;
    VIEW_CUDA(ctx, cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    cudaError_t e = cudaEventRecord(ev, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, ev, 0);
    if (e == cudaSuccess)
        e = gr::filter_rgba8((const double*)sc->fb.p, (const uint32_t*)sc->fb_count.p, sc->cam.width * sc->cam.height,
                             d_rgba, s);
    cudaEventDestroy(ev);
    return view_cuda(ctx, e, "gr_scene_rgba8");
}

gr_status gr_scene_rgba8_host(gr_scene* sc, uint32_t* h_rgba) {
    if (!sc || !h_rgba) return GR_ERR_INVALID;
    gr_ctx* ctx = sc->ctx;
    VIEW_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t npix = (size_t)sc->cam.width * sc->cam.height;
    VIEW_CUDA(ctx, ctx->stage_out.ensure(4 * npix));
    const gr_status st = gr_scene_rgba8(sc, (uint32_t*)ctx->stage_out.p, ctx->stream);
    if (st != GR_OK) return st;
    VIEW_CUDA(ctx, cudaMemcpyAsync(h_rgba, ctx->stage_out.p, 4 * npix, cudaMemcpyDeviceToHost, ctx->stream));
    VIEW_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return GR_OK;
}

}  // extern "C"
