// Batched rendering and the render server (include/gr.h). The reference has
// no counterpart: it renders one scene, one sample per call.
//
// Both drive the same wave machinery as gr_render (render.cu): jobs are packed
// into waves of at most `capacity` paths, each wave's job table is staged and
// the captured wave is replayed. Because a path's result depends only on its
// scene, pixel and sample, and each job's pixels are resolved in sample order,
// a job's image is identical whatever else shares its waves.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "render.h"

namespace {

gr_status cuda_status(cudaError_t e) { return e == cudaErrorMemoryAllocation ? GR_ERR_OOM_BUDGET : GR_ERR_CUDA; }

// the server's pool when its options leave the wave size open
uint32_t default_capacity(uint32_t wave_paths) { return wave_paths ? wave_paths : (1u << 22); }

}  // namespace

gr::WavePool* gr::context_pool(gr_ctx* ctx) {
    if (!ctx->batch_pool) {
        ctx->batch_pool = new (std::nothrow) gr::WavePool();
        if (!ctx->batch_pool) return nullptr;
        ctx->batch_pool_free = [](void* p) { delete static_cast<gr::WavePool*>(p); };
    }
    return static_cast<gr::WavePool*>(ctx->batch_pool);
}

namespace {

// Per-pixel mean of an accumulation (for the server's results).
void mean_image(const double* sum, const uint32_t* cnt, uint32_t npix, float* out) {
    for (uint32_t p = 0; p < npix; ++p) {
        const double inv = cnt[p] ? 1.0 / cnt[p] : 0.0;
        for (int c = 0; c < 3; ++c) out[3ull * p + c] = (float)(sum[3ull * p + c] * inv);
    }
}

}  // namespace

extern "C" uint64_t gr_scene_device_bytes(const gr_scene* sc) {
    if (!sc) return 0;
    uint64_t b = sc->verts.bytes + sc->normals.bytes + sc->tri_mat.bytes + sc->mats.bytes + sc->lights.bytes +
                 sc->uvs.bytes + sc->texels.bytes + sc->env_map.bytes +
                 sc->fb.bytes + sc->fb_count.bytes;
    if (sc->bvh) {
        const gr::BvhBuffers& bb = sc->bvh->buf;
        b += bb.nodes.bytes + bb.nodes4.bytes + bb.nodes4q.bytes + bb.nodes8.bytes + bb.tris8.bytes + bb.tris.bytes +
             bb.code.bytes + bb.prim.bytes + bb.scratch.bytes + bb.meta.bytes;
    }
    return b;
}

extern "C" gr_status gr_render_batch(gr_ctx* ctx, gr_scene* const* scenes, const gr_render_opts* opts, uint32_t n,
                                     uint32_t wave_paths, gr_render_stats* stats) {
    if (!ctx || (n && (!scenes || !opts))) return GR_ERR_INVALID;
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<gr::HostJob> jobs(n);
    std::vector<gr::HostJob*> order;
    uint32_t max_npix = 1;
    for (uint32_t i = 0; i < n; ++i) {
        gr_scene* sc = scenes[i];
        if (!sc || sc->ctx != ctx || opts[i].max_depth > (uint32_t)gr::kMaxDepth) {
            ctx->last_error = "gr_render_batch: bad job " + std::to_string(i);
            return GR_ERR_INVALID;
        }
        for (uint32_t k = 0; k < i; ++k)
            if (scenes[k] == sc) {
                ctx->last_error = "gr_render_batch: a scene appears twice";
                return GR_ERR_INVALID;
            }
        if (sc->bvh->layout != scenes[0]->bvh->layout) {
            ctx->last_error = "gr_render_batch: scenes use different node layouts";
            return GR_ERR_INVALID;
        }
        gr::HostJob& j = jobs[i];
        j.sc = gr::scene_view(sc, sc->bvh->layout);
        j.fb = (double*)sc->fb.p;
        j.fbc = (uint32_t*)sc->fb_count.p;
        j.npix = sc->cam.width * sc->cam.height;
        j.spp_total = opts[i].spp;
        j.spp_done = 0;
        j.sample_offset = sc->samples_done;
        j.max_depth = opts[i].max_depth;
        j.rr_depth = opts[i].rr_depth;
        j.flags = opts[i].flags;
        j.seed = opts[i].seed;
        order.push_back(&j);
        max_npix = std::max(max_npix, j.npix);
    }
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_status(e);
    uint64_t want = wave_paths ? wave_paths : ctx->default_wave_paths;
    uint64_t work = 0;
    for (uint32_t i = 0; i < n; ++i) work += (uint64_t)opts[i].spp * jobs[i].npix;
    want = std::min<uint64_t>(want, std::max<uint64_t>(work, 1));  // no larger than the batch
    gr::WavePool* pp = gr::context_pool(ctx);
    if (!pp) return GR_ERR_OOM_BUDGET;
    gr::WavePool& pool = *pp;
    // the default wave halves until the device has room for it
    uint32_t cap = (uint32_t)std::max<uint64_t>(want, max_npix);
    while ((e = pool.ensure(cap)) != cudaSuccess && !wave_paths && cap / 2 >= max_npix) {
        cudaGetLastError();
        cap /= 2;
    }
    if (e != cudaSuccess) {
        ctx->last_error = std::string("gr_render_batch: ") + cudaGetErrorString(e);
        return cuda_status(e);
    }
    cudaStream_t s = ctx->stream;
    if ((e = pool.clear_errors(s)) != cudaSuccess) return cuda_status(e);
    gr::WaveHeader before{};
    cudaMemcpyAsync(&before, pool.ps.hdr, sizeof(before), cudaMemcpyDeviceToHost, s);
    std::vector<gr::JobDev> table;
    uint32_t waves = 0;
    const bool graph = !(n && (opts[0].flags & GR_RENDER_NO_GRAPH));
    for (;;) {
        uint32_t paths = 0, pix = 0, depth = 0;
        // the requested wave size, not a larger pool an earlier call left behind
        const uint32_t nj = gr::pack_wave(order, cap, table, &paths, &pix, &depth);
        if (nj == 0) break;
        if ((e = gr::run_wave(pool, table.data(), nj, paths, pix, depth, ctx->num_sms, s, graph,
                              scene_tuning(scenes[0]))) != cudaSuccess) {
            ctx->last_error = std::string("gr_render_batch: ") + cudaGetErrorString(e);
            cudaGetLastError();
            return cuda_status(e);
        }
        ++waves;
    }
    gr::WaveHeader after{};
    uint32_t err = 0;
    cudaMemcpyAsync(&after, pool.ps.hdr, sizeof(after), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&err, pool.error_word(), 4, cudaMemcpyDeviceToHost, s);
    if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_status(e);
    uint64_t samples = 0;
    for (uint32_t i = 0; i < n; ++i) {
        scenes[i]->samples_done += opts[i].spp;
        samples += (uint64_t)opts[i].spp * jobs[i].npix;
    }
    if (stats) {
        stats->ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        stats->closest_rays = after.closest_rays - before.closest_rays;
        stats->shadow_rays = after.shadow_rays - before.shadow_rays;
        stats->samples = samples;
        stats->waves = waves;
        stats->device_errors = err;
    }
    if (err) {
        ctx->last_error = "gr_render_batch: device error bits set";
        return (err & gr::ERR_STACK) ? GR_ERR_OVERFLOW : GR_ERR_CUDA;
    }
    return GR_OK;
}

// ---- server ---------------------------------------------------------------------------------

namespace {

// Free lists of device and pinned host buffers by size, so jobs coming and
// going do not call cudaMalloc / cudaFree (which would synchronise the device)
// once the pool is warm.
struct BufCache {
    std::multimap<size_t, void*> dev_free, host_free;
    void* get_dev(size_t bytes, cudaError_t* e) {
        auto it = dev_free.find(bytes);
        if (it != dev_free.end()) {
            void* p = it->second;
            dev_free.erase(it);
            return p;
        }
        void* p = nullptr;
        *e = cudaMalloc(&p, bytes);
        return *e == cudaSuccess ? p : nullptr;
    }
    void* get_host(size_t bytes, cudaError_t* e) {
        auto it = host_free.find(bytes);
        if (it != host_free.end()) {
            void* p = it->second;
            host_free.erase(it);
            return p;
        }
        void* p = nullptr;
        *e = cudaMallocHost(&p, bytes);
        return *e == cudaSuccess ? p : nullptr;
    }
    void put_dev(size_t bytes, void* p) { dev_free.emplace(bytes, p); }
    void put_host(size_t bytes, void* p) { host_free.emplace(bytes, p); }
    void clear() {
        for (auto& kv : dev_free) cudaFree(kv.second);
        for (auto& kv : host_free) cudaFreeHost(kv.second);
        dev_free.clear();
        host_free.clear();
    }
};

struct Job {
    uint64_t ticket = 0;
    gr_scene* scene = nullptr;
    gr_render_opts opts{};
    gr::HostJob hj{};
    double* d_sum = nullptr;
    uint32_t* d_cnt = nullptr;
    void* h_res = nullptr;  // pinned: sums then counts
    size_t dev_bytes = 0, host_bytes = 0;
    cudaEvent_t done_ev = nullptr;
    uint32_t waves = 0;
    uint64_t first_wave = 0, last_wave = 0;
    bool scheduled_all = false;
    bool finished = false;
    std::vector<float> image;
    gr_job_stats st{};
};

}  // namespace

struct gr_server {
    gr_ctx* ctx = nullptr;
    gr_server_opts opts{};
    cudaStream_t stream = nullptr;
    gr::WavePool pool;
    BufCache cache;
    std::thread worker;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    bool stop = false;
    uint64_t next_ticket = 1;
    std::deque<std::shared_ptr<Job>> pending;
    std::vector<std::shared_ptr<Job>> active;
    std::unordered_map<uint64_t, std::shared_ptr<Job>> all;
    std::unordered_map<gr_scene*, int> scene_refs;
    uint64_t bytes_in_use = 0;
    double busy_since = -1.0;       // server clock when the current busy period began (-1: idle)
    uint64_t paths_retired = 0;     // paths of completed jobs (throughput estimate)
    std::atomic<uint32_t> inject_wave_failures{0};
    gr_server_stats stats{};
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    std::string error;

    double now() const { return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count(); }

    uint64_t job_bytes(const Job& j) const { return (uint64_t)j.hj.npix * (24 + 4); }

    // Paths (pixels x samples) a job has not yet scheduled.
    static uint64_t remaining(const Job& j) { return (uint64_t)(j.hj.spp_total - j.hj.spp_done) * j.hj.npix; }

    // GR_SERVER_SHORTEST_FIRST order: jobs older than the age cap first (oldest
    // first), then the least remaining work first (ties by arrival). Returns
    // true when a goes before b.
    bool before(const Job& a, const Job& b, double t) const {
        const bool aged_a = opts.age_cap_s > 0 && t - a.st.submit_s > opts.age_cap_s;
        const bool aged_b = opts.age_cap_s > 0 && t - b.st.submit_s > opts.age_cap_s;
        if (aged_a != aged_b) return aged_a;
        if (aged_a) return a.ticket < b.ticket;
        const uint64_t ra = remaining(a), rb = remaining(b);
        return ra != rb ? ra < rb : a.ticket < b.ticket;
    }

    // Measured throughput (paths per second of busy time) and the paths queued
    // or running, for load shedding (with mu held).
    double busy_seconds() const { return stats.busy_s + (busy_since >= 0 ? now() - busy_since : 0.0); }
    uint64_t queued_paths() const {
        uint64_t q = 0;
        for (const auto& j : pending) q += remaining(*j);
        for (const auto& j : active) q += remaining(*j);
        return q;
    }

    // Admission under the budget (called with mu held).
    void admit() {
        const uint32_t max_active = opts.max_active ? opts.max_active : gr::kMaxJobs;
        while (!pending.empty() && active.size() < max_active) {
            if (opts.policy == GR_SERVER_SHORTEST_FIRST) {  // the next job to admit goes to the front
                const double t = now();
                auto best = pending.begin();
                for (auto it = pending.begin() + 1; it != pending.end(); ++it)
                    if (before(**it, **best, t)) best = it;
                if (best != pending.begin()) std::iter_swap(pending.begin(), best);
            }
            Job& j = *pending.front();
            uint64_t need = job_bytes(j);
            if (!scene_refs.count(j.scene)) need += gr_scene_device_bytes(j.scene);
            if (opts.budget_bytes && bytes_in_use + need > opts.budget_bytes && !active.empty()) break;
            cudaError_t e = cudaSuccess;
            j.dev_bytes = job_bytes(j);
            char* d = (char*)cache.get_dev(j.dev_bytes, &e);
            j.host_bytes = j.dev_bytes;
            void* h = d ? cache.get_host(j.host_bytes, &e) : nullptr;
            if (!d || !h) {
                if (d) cache.put_dev(j.dev_bytes, d);
                j.st.status = cuda_status(e);
                j.finished = true;
                j.st.done_s = now();
                pending.pop_front();
                cv_done.notify_all();
                continue;
            }
            j.d_sum = (double*)d;
            j.d_cnt = (uint32_t*)(d + 24ull * j.hj.npix);
            j.h_res = h;
            j.hj.fb = j.d_sum;
            j.hj.fbc = j.d_cnt;
            e = cudaMemsetAsync(d, 0, j.dev_bytes, stream);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&j.done_ev, cudaEventDisableTiming);
            if (e != cudaSuccess) {  // the job fails; nothing of it is in flight
                cudaGetLastError();
                cache.put_dev(j.dev_bytes, d);
                cache.put_host(j.host_bytes, h);
                j.d_sum = nullptr;
                j.h_res = nullptr;
                j.done_ev = nullptr;
                error = cudaGetErrorString(e);
                j.st.status = cuda_status(e);
                j.finished = true;
                j.st.done_s = now();
                pending.pop_front();
                cv_done.notify_all();
                continue;
            }
            j.st.admit_s = now();
            scene_refs[j.scene]++;
            bytes_in_use += need;
            stats.peak_bytes = std::max(stats.peak_bytes, bytes_in_use);
            stats.admitted++;
            active.push_back(pending.front());
            pending.pop_front();
        }
    }

    void release_job(Job& j) {  // with mu held
        cache.put_dev(j.dev_bytes, j.d_sum);
        cache.put_host(j.host_bytes, j.h_res);
        uint64_t freed = job_bytes(j);
        if (--scene_refs[j.scene] == 0) {
            scene_refs.erase(j.scene);
            freed += gr_scene_device_bytes(j.scene);
        }
        bytes_in_use -= std::min(bytes_in_use, freed);
        if (j.done_ev) cudaEventDestroy(j.done_ev);
        j.done_ev = nullptr;
    }

    // Ends an active job with an error status (with mu held): its buffers go
    // back to the free lists (later work on the server's stream is ordered
    // after anything still queued for it) and its waiters are woken.
    void fail_active(const std::shared_ptr<Job>& j, gr_status st) {
        if (j->finished) return;
        j->st.status = st;
        j->st.done_s = now();
        j->finished = true;
        release_job(*j);
        auto it = std::find(active.begin(), active.end(), j);
        if (it != active.end()) active.erase(it);
        cv_done.notify_all();
    }

    void run() {
        cudaSetDevice(ctx->device);
        std::vector<gr::JobDev> table;
        for (;;) {
            std::vector<std::shared_ptr<Job>> act;
            std::vector<Job*> order;
            std::vector<uint32_t> done_before;
            uint32_t nj = 0, paths = 0, pix = 0, depth = 0;
            {
                std::unique_lock<std::mutex> lk(mu);
                admit();
                if (active.empty()) {
                    if (busy_since >= 0) {
                        stats.busy_s += now() - busy_since;
                        busy_since = -1.0;
                    }
                    if (stop) break;
                    cv_work.wait_for(lk, std::chrono::milliseconds(2));
                    continue;
                }
                if (busy_since < 0) busy_since = now();
                act = active;
                // pack one wave over the active jobs that still need samples, in
                // the policy's order (under the lock: submit reads the progress)
                for (auto& j : act)
                    if (!j->scheduled_all) order.push_back(j.get());
                if (opts.policy == GR_SERVER_SHORTEST_FIRST) {
                    const double t = now();
                    std::stable_sort(order.begin(), order.end(),
                                     [&](const Job* a, const Job* b) { return before(*a, *b, t); });
                }
                std::vector<gr::HostJob*> hjs;
                for (Job* j : order) {
                    hjs.push_back(&j->hj);
                    done_before.push_back(j->hj.spp_done);
                }
                if (!hjs.empty()) nj = gr::pack_wave(hjs, pool.capacity, table, &paths, &pix, &depth);
            }
            if (!order.empty()) {
                if (nj) {
                    gr::TraceTuning tune;
                    tune.layout = opts.layout;
                    tune.block = opts.block;
                    tune.sstack = opts.short_stack;
                    cudaError_t e;
                    if (inject_wave_failures.load() > 0) {  // host-side fault injection (gr_diag_server_fail_waves)
                        inject_wave_failures.fetch_sub(1);
                        e = cudaErrorLaunchFailure;
                    } else {
                        e = gr::run_wave(pool, table.data(), nj, paths, pix, depth, ctx->num_sms, stream, true, tune);
                    }
                    std::lock_guard<std::mutex> lk(mu);
                    if (e != cudaSuccess) {
                        // every job in flight fails: its samples cannot be completed
                        cudaGetLastError();
                        error = cudaGetErrorString(e);
                        for (auto& j : act) fail_active(j, cuda_status(e));
                        continue;
                    }
                    stats.waves++;
                    for (size_t k = 0; k < order.size(); ++k) {  // the jobs this wave carried
                        if (order[k]->hj.spp_done == done_before[k]) continue;
                        Job& j = *order[k];
                        if (!j.first_wave) j.first_wave = stats.waves;
                        j.last_wave = stats.waves;
                        j.waves++;
                    }
                }
                // jobs whose last samples went into this wave: copy out after it
                for (auto& j : act) {
                    if (j->scheduled_all || j->hj.spp_done < j->hj.spp_total) continue;
                    j->scheduled_all = true;
                    const size_t npix = j->hj.npix;
                    cudaError_t ce = cudaMemcpyAsync(j->h_res, j->d_sum, 28 * npix, cudaMemcpyDeviceToHost, stream);
                    if (ce == cudaSuccess) ce = cudaEventRecord(j->done_ev, stream);
                    if (ce != cudaSuccess) {
                        cudaGetLastError();
                        std::lock_guard<std::mutex> lk(mu);
                        error = cudaGetErrorString(ce);
                        fail_active(j, cuda_status(ce));
                    }
                }
            } else {
                std::this_thread::sleep_for(std::chrono::microseconds(50));
            }
            // retire finished jobs
            for (auto& j : act) {
                if (!j->scheduled_all || j->finished) continue;
                const cudaError_t q = cudaEventQuery(j->done_ev);
                if (q == cudaErrorNotReady) continue;
                if (q != cudaSuccess) {  // an error, not completion: the job fails instead of waiting forever
                    cudaGetLastError();
                    std::lock_guard<std::mutex> lk(mu);
                    error = cudaGetErrorString(q);
                    fail_active(j, cuda_status(q));
                    continue;
                }
                const uint32_t npix = j->hj.npix;
                j->image.resize(3ull * npix);
                const double* sum = (const double*)j->h_res;
                const uint32_t* cnt = (const uint32_t*)((const char*)j->h_res + 24ull * npix);
                mean_image(sum, cnt, npix, j->image.data());
                std::lock_guard<std::mutex> lk(mu);
                j->st.done_s = now();
                j->st.samples = (uint64_t)j->hj.spp_total * npix;
                paths_retired += j->st.samples;
                j->finished = true;
                release_job(*j);
                active.erase(std::find(active.begin(), active.end(), j));
                stats.completed++;
                cv_done.notify_all();
            }
        }
        cudaStreamSynchronize(stream);
    }
};

extern "C" {

gr_status gr_server_create(gr_ctx* ctx, const gr_server_opts* opts, gr_server** out) {
    if (!ctx || !out) return GR_ERR_INVALID;
    *out = nullptr;
    gr_server* sv = new (std::nothrow) gr_server();
    if (!sv) return GR_ERR_OOM_BUDGET;
    sv->ctx = ctx;
    if (opts) sv->opts = *opts;
    if (!sv->opts.block) sv->opts.block = 128;
    if (!sv->opts.short_stack) sv->opts.short_stack = 12;
    gr::TraceTuning tt;
    tt.layout = sv->opts.layout;
    tt.block = sv->opts.block;
    tt.sstack = sv->opts.short_stack;
    if (!gr::tuning_valid(tt)) {
        ctx->last_error = "gr_server_create: unsupported layout / block / short_stack";
        delete sv;
        return GR_ERR_INVALID;
    }
    if ((sv->opts.policy != GR_SERVER_FIFO && sv->opts.policy != GR_SERVER_SHORTEST_FIRST) ||
        !(sv->opts.age_cap_s >= 0) || !(sv->opts.max_wait_s >= 0)) {
        ctx->last_error = "gr_server_create: unknown policy or negative age cap / wait limit";
        delete sv;
        return GR_ERR_INVALID;
    }
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&sv->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = sv->pool.ensure(default_capacity(sv->opts.wave_paths));
    if (e != cudaSuccess) {
        ctx->last_error = std::string("gr_server_create: ") + cudaGetErrorString(e);
        sv->pool.release();
        if (sv->stream) cudaStreamDestroy(sv->stream);
        delete sv;
        return cuda_status(e);
    }
    sv->bytes_in_use = sv->pool.mem.bytes;
    sv->stats.peak_bytes = sv->bytes_in_use;
    gr::ctx_retain(ctx);
    sv->worker = std::thread([sv] { sv->run(); });
    *out = sv;
    return GR_OK;
}

gr_status gr_server_destroy(gr_server* sv) {
    if (!sv) return GR_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
        sv->pending.clear();
    }
    sv->cv_work.notify_all();
    sv->worker.join();
    gr_ctx* ctx = sv->ctx;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(sv->stream);
    for (auto& kv : sv->all)
        if (kv.second->done_ev) cudaEventDestroy(kv.second->done_ev);
    sv->pool.release();
    sv->cache.clear();
    cudaStreamDestroy(sv->stream);
    delete sv;
    gr::ctx_release(ctx);
    return GR_OK;
}

double gr_server_now(const gr_server* sv) { return sv ? sv->now() : 0.0; }

gr_status gr_diag_server_fail_waves(gr_server* sv, uint32_t count) {
    if (!sv) return GR_ERR_INVALID;
    sv->inject_wave_failures.store(count);
    return GR_OK;
}

gr_status gr_server_submit(gr_server* sv, gr_scene* scene, const gr_camera* camera, const gr_render_opts* opts,
                           uint64_t* ticket) {
    if (!sv || !scene || !opts || !ticket || scene->ctx != sv->ctx) return GR_ERR_INVALID;
    if (opts->max_depth > (uint32_t)gr::kMaxDepth) return GR_ERR_INVALID;
    // the scene must have the server's node layout built before it joins a wave
    if (scene->bvh->layout != sv->opts.layout || !scene->bvh->built) {
        gr_status st = gr_scene_set_layout(scene, sv->opts.layout);
        if (st != GR_OK) return st;
    }
    gr::SceneDev view = gr::scene_view(scene, sv->opts.layout);
    if (camera) {
        if (!gr::pixels_ok(camera->width, camera->height) || !(camera->fov_deg > 0.0f && camera->fov_deg < 180.0f))
            return GR_ERR_INVALID;
        view.cam = gr::make_camera(*camera);
    }
    const uint64_t npix64 = (uint64_t)view.cam.width * view.cam.height;
    if (npix64 > sv->pool.capacity) return GR_ERR_INVALID;  // a job's pixels must fit one wave
    const uint32_t npix = (uint32_t)npix64;
    auto j = std::make_shared<Job>();
    j->scene = scene;
    j->opts = *opts;
    j->hj.sc = view;
    j->hj.npix = npix;
    j->hj.spp_total = opts->spp;
    j->hj.spp_done = 0;
    j->hj.sample_offset = 0;
    j->hj.max_depth = opts->max_depth;
    j->hj.rr_depth = opts->rr_depth;
    j->hj.flags = opts->flags;
    j->hj.seed = opts->seed;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (sv->opts.max_wait_s > 0) {  // load shedding at the measured throughput
            const double busy = sv->busy_seconds();
            if (sv->paths_retired > 0 && busy > 0) {
                const double rate = (double)sv->paths_retired / busy;
                const double wait = (double)(sv->queued_paths() + (uint64_t)npix * opts->spp) / rate;
                if (wait > sv->opts.max_wait_s) {
                    sv->stats.rejected++;
                    return GR_ERR_BUSY;
                }
            }
        }
        j->ticket = sv->next_ticket++;
        j->st.submit_s = sv->now();
        sv->pending.push_back(j);
        sv->all[j->ticket] = j;
        sv->stats.submitted++;
        *ticket = j->ticket;
    }
    sv->cv_work.notify_all();
    return GR_OK;
}

gr_status gr_server_wait(gr_server* sv, uint64_t ticket, double timeout_s, int* done, float* h_rgb,
                         gr_job_stats* stats) {
    if (!sv) return GR_ERR_INVALID;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->all.find(ticket);
    if (it == sv->all.end()) return GR_ERR_INVALID;
    std::shared_ptr<Job> j = it->second;
    auto pred = [&] { return j->finished; };
    if (timeout_s < 0) sv->cv_done.wait(lk, pred);
    else sv->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred);
    if (done) *done = j->finished ? 1 : 0;
    j->st.waves = j->waves;
    j->st.first_wave = j->first_wave;
    j->st.last_wave = j->last_wave;
    if (stats) *stats = j->st;
    if (j->finished && h_rgb && !j->image.empty()) std::memcpy(h_rgb, j->image.data(), j->image.size() * 4);
    if (j->finished) {
        sv->all.erase(it);  // a finished job is reported once
        return (gr_status)j->st.status;
    }
    return GR_OK;
}

gr_status gr_server_poll(gr_server* sv, uint64_t ticket, int* done, float* h_rgb, gr_job_stats* stats) {
    return gr_server_wait(sv, ticket, 0.0, done, h_rgb, stats);
}

gr_status gr_server_stats_get(gr_server* sv, gr_server_stats* out) {
    if (!sv || !out) return GR_ERR_INVALID;
    gr::WaveHeader h{};
    cudaSetDevice(sv->ctx->device);
    // ray totals live in the pool's device header
    cudaMemcpyAsync(&h, sv->pool.ps.hdr, sizeof(h), cudaMemcpyDeviceToHost, sv->stream);
    cudaStreamSynchronize(sv->stream);
    std::lock_guard<std::mutex> lk(sv->mu);
    *out = sv->stats;
    out->closest_rays = h.closest_rays;
    out->shadow_rays = h.shadow_rays;
    out->bytes_in_use = sv->bytes_in_use;
    return GR_OK;
}

}  // extern "C"
