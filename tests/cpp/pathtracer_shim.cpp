// A consumer of include/gr.h written the way a maintainer of the reference
// would keep its API: the reference's PathTracer class
// (src/renderer/pathtracer.h:16-46; render(num) pathtracer.cu:152-170,
// output pathtracer.cu:172-175, reset/zoom/rotate pathtracer.cu:177-213) as a
// thin C++ class over the C ABI. The wavefront loop, queues, BVH and
// framebuffer all live in libgr.so.
//
// Usage: pathtracer_shim <scene.xml> <frames> <max_depth> <seed> <out.pfm|out.png>
// Renders `frames` one-sample frames progressively (the reference's main loop),
// writes the image and prints one line: width height samples closest_rays.
#include <cstdio>
#include <cstdlib>
#include <stdexcept>
#include <string>
#include <vector>

#include "gr.h"

class PathTracer {
  public:
    explicit PathTracer(const std::string& xml, uint32_t max_depth, uint64_t seed)
        : max_depth_(max_depth), seed_(seed) {
        gr_opts opts{};  // library defaults
        if (gr_context_create(0, &opts, &ctx_) != GR_OK) throw std::runtime_error("no CUDA device / context");
        check(gr_scene_load_xml(ctx_, xml.c_str(), &scene_));
        uint32_t tris = 0, lights = 0;
        check(gr_scene_info(scene_, &w_, &h_, &tris, &lights));
    }
    ~PathTracer() {
        if (scene_) gr_scene_destroy(scene_);
        if (ctx_) gr_context_destroy(ctx_);
    }
    PathTracer(const PathTracer&) = delete;
    PathTracer& operator=(const PathTracer&) = delete;

    // render(uint32 num): num more samples per pixel; the running mean is kept
    void render(uint32_t num) {
        gr_render_opts o{};
        o.spp = num;
        o.max_depth = max_depth_;
        o.seed = seed_;
        o.rr_depth = 3;  // roulette after bounce 3 (pathtracer_kernel.h:738)
        o.flags = 0;
        o.wave_paths = 0;
        rgb_.resize(3ull * w_ * h_);
        gr_render_stats st{};
        check(gr_render(scene_, &o, rgb_.data(), &st));
        samples_ += st.samples;
        closest_rays_ += st.closest_rays;
    }
    void output(const std::string& path) { check(gr_scene_write_image(scene_, path.c_str())); }
    void reset() { check(gr_scene_reset(scene_)); }
    void zoom(float d) { check(gr_scene_zoom(scene_, d)); }
    void rotate(float yaw, float pitch) { check(gr_scene_rotate(scene_, yaw, pitch)); }

    uint32_t width() const { return w_; }
    uint32_t height() const { return h_; }
    uint64_t samples() const { return samples_; }
    uint64_t closest_rays() const { return closest_rays_; }
    const std::vector<float>& image() const { return rgb_; }

  private:
    void check(gr_status s) {
        if (s != GR_OK) throw std::runtime_error(std::string(gr_status_string(s)) + ": " + gr_last_error(ctx_));
    }
    gr_ctx* ctx_ = nullptr;
    gr_scene* scene_ = nullptr;
    uint32_t w_ = 0, h_ = 0;
    uint32_t max_depth_;
    uint64_t seed_;
    uint64_t samples_ = 0, closest_rays_ = 0;
    std::vector<float> rgb_;
};

int main(int argc, char** argv) {
    if (argc != 6) {
        std::fprintf(stderr, "usage: %s scene.xml frames max_depth seed out.pfm\n", argv[0]);
        return 2;
    }
    try {
        PathTracer pt(argv[1], (uint32_t)std::atoi(argv[3]), (uint64_t)std::strtoull(argv[4], nullptr, 10));
        const int frames = std::atoi(argv[2]);
        for (int f = 0; f < frames; ++f) pt.render(1);
        pt.output(argv[5]);
        std::printf("%u %u %llu %llu\n", pt.width(), pt.height(), (unsigned long long)pt.samples(),
                    (unsigned long long)pt.closest_rays());
    } catch (const std::exception& e) {
        std::fprintf(stderr, "pathtracer_shim: %s\n", e.what());
        return 1;
    }
    return 0;
}
