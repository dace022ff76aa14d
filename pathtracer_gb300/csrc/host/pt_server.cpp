// pt_server.cpp — the render-serving loop (pt_host.h, pt_server_*).
//
// No counterpart in the reference, whose host renders one scene at a time
// (src/pathtracer.cpp:3965-4093).  Requests name a resident scene and ask
// for a target error; the server refines each admitted job with progressive
// passes of the reference's method until its relative RMSE against the
// scene's FP64 reference reaches the target (or a sample cap), and reports
// queueing and completion times.
//
//   PT_SERVE_BATCHED  continuous batching: requests are admitted FIFO while
//                     their accumulator and in-flight sample colours fit the
//                     HBM budget; every admitted job keeps one pass in flight
//                     in a shared pt_batch, so passes of many jobs run in the
//                     same launches; RMSE checks of all jobs whose pass
//                     finished are one reduction.
//   PT_SERVE_PLAIN    the drop-in path: one job at a time through pt_dispatch
//                     on the plain megakernel, an RMSE check after each pass.
//
// Pass k (1-based) of a job renders samples [(k-1)*spf, k*spf) with
// frame = currentSamples = k*spf, exactly the reference's offscreen
// progressive loop, so a job's image after k passes is bit-identical in both
// modes and whatever else is in flight.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../../include/pt_host.h"

namespace {

struct SceneEntry {
    int batch_scene = -1;
    pt_ubo* ubo = nullptr;  // host copy for the plain path's uploads
    std::vector<pt_sdf_plugin> plugins;
    std::vector<std::string> sources;  // SDF texts (scenes added with sources)
    std::shared_ptr<pt_scene_ext> ext;  // full-form extensions (null: the reference's method)
    int ref_target = -1;
    int ref_w = 0, ref_h = 0;
};

struct Job {
    uint64_t id = 0;
    pt_server_job req{};
    int width = 0, height = 0;
    int spf = 8;
    int target = -1;           // batched mode
    int passes_done = 0;
    int passes_in_flight = 0;
    int last_pass = -1;
    double rmse = -1.0;
    double t_submit = 0, t_admit = -1, t_done = -1;
    uint64_t bytes = 0;
    bool finished = false;
    int status = PT_OK;
};

}  // namespace

struct pt_server {
    pt_server_opts opts{};
    int device = 0;
    pt_batch* batch = nullptr;
    pt_ctx* ctx = nullptr;  // plain mode
    int ctx_scene = -1, ctx_w = 0, ctx_h = 0;
    std::map<int, SceneEntry> scenes;
    std::unordered_map<uint64_t, Job> jobs;
    std::deque<uint64_t> queue;   // submitted, not admitted (FIFO)
    std::vector<uint64_t> active; // admitted, not finished
    std::unordered_map<int, uint64_t> pass_job;  // batch pass id -> job
    uint64_t next_id = 1;
    uint64_t bytes_in_use = 0, bytes_peak = 0, resident_bytes = 0;
    uint64_t submitted = 0, admitted = 0, completed = 0, samples = 0;
    std::chrono::steady_clock::time_point t0;
    std::string err;
    std::vector<pt_server_result> ready;  // finished, not yet returned by poll
};

namespace {

int sfail(pt_server* s, int code, const std::string& msg) {
    s->err = msg;
    return code;
}

int from_batch(pt_server* s, int rc, const char* what) {
    if (rc != PT_OK) s->err = std::string(what) + ": " + pt_batch_last_error(s->batch);
    return rc;
}

int from_ctx(pt_server* s, int rc, const char* what) {
    if (rc != PT_OK) s->err = std::string(what) + ": " + pt_last_error(s->ctx);
    return rc;
}

double now_s(const pt_server* s) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - s->t0).count();
}

pt_push pass_push(const Job& j, int k) {
    pt_push p = j.req.push;
    p.samplesPerFrame = j.spf;
    p.frame = k * j.spf;
    p.currentSamples = k * j.spf;
    return p;
}

// Bytes an admitted job holds: its accumulator and the sample colours of its
// passes in flight.
uint64_t job_bytes(const pt_server* s, const Job& j) {
    const uint64_t px = (uint64_t)j.width * (uint64_t)j.height;
    return px * 16ull + px * 16ull * (uint64_t)j.spf * (uint64_t)s->opts.passes_in_flight;
}

bool done_with(const Job& j) {
    if (j.status == PT_ERR_CANCELLED) return true;
    const int spp = j.passes_done * j.spf;
    if (j.req.target_rmse > 0.0 && j.rmse >= 0.0 && j.rmse <= j.req.target_rmse) return true;
    return spp >= j.req.max_spp;
}

void finish(pt_server* s, Job& j, double t) {
    j.finished = true;
    j.t_done = t;
    pt_server_result r{};
    r.job_id = j.id;
    r.status = j.status;
    r.spp = j.passes_done * j.spf;
    r.rmse = j.rmse;
    r.t_submit = j.t_submit;
    r.t_admit = j.t_admit;
    r.t_done = j.t_done;
    r.samples = (uint64_t)j.width * (uint64_t)j.height * (uint64_t)r.spp;
    s->samples += r.samples;
    s->completed++;
    s->ready.push_back(r);
    if (!s->opts.keep_images && j.target >= 0) {
        pt_batch_release_target(s->batch, j.target);
        j.target = -1;
    }
    if (s->opts.mode == PT_SERVE_BATCHED) s->bytes_in_use -= j.bytes;
}

// ---- batched mode -----------------------------------------------------------

int admit_batched(pt_server* s, double t) {
    while (!s->queue.empty()) {
        Job& j = s->jobs[s->queue.front()];
        const uint64_t b = job_bytes(s, j);
        if (!s->active.empty() && s->bytes_in_use + b > s->opts.hbm_budget) break;  // FIFO: wait for memory
        int rc = pt_batch_add_target(s->batch, j.width, j.height, PT_TARGET_FLOAT, &j.target);
        if (rc != PT_OK) return from_batch(s, rc, "admit");
        j.bytes = b;
        j.t_admit = t;
        s->bytes_in_use += b;
        s->bytes_peak = std::max(s->bytes_peak, s->bytes_in_use);
        s->admitted++;
        s->active.push_back(j.id);
        s->queue.pop_front();
    }
    return PT_OK;
}

int feed_batched(pt_server* s) {
    for (uint64_t id : s->active) {
        Job& j = s->jobs[id];
        while (!j.finished && j.status == PT_OK && j.passes_in_flight < s->opts.passes_in_flight &&
               (j.passes_done + j.passes_in_flight) * j.spf < j.req.max_spp) {
            const SceneEntry& sc = s->scenes[j.req.scene_key];
            const pt_push p = pass_push(j, j.passes_done + j.passes_in_flight + 1);
            int pid = -1;
            const int rc = pt_batch_add_pass(s->batch, sc.batch_scene, j.target, &p, &pid);
            if (rc == PT_ERR_BUSY) return PT_OK;  // ring full: more next round
            if (rc != PT_OK) return from_batch(s, rc, "pass");
            j.passes_in_flight++;
            j.last_pass = pid;
            s->pass_job[pid] = id;
        }
    }
    return PT_OK;
}

int poll_batched(pt_server* s) {
    int rc = admit_batched(s, now_s(s));
    if (rc != PT_OK) return rc;
    rc = feed_batched(s);
    if (rc != PT_OK) return rc;
    if (s->active.empty()) return PT_OK;
    std::vector<int> ids(4096);
    int n = 0;
    rc = pt_batch_step(s->batch, s->opts.iterations_per_poll, ids.data(), (int)ids.size(), &n);
    if (rc != PT_OK) return from_batch(s, rc, "step");
    if (n == 0) return PT_OK;
    // Jobs whose newest resolved pass needs an error check.
    std::vector<uint64_t> check;
    std::vector<int> tgt, ref;
    for (int i = 0; i < n; i++) {
        auto it = s->pass_job.find(ids[(size_t)i]);
        if (it == s->pass_job.end()) continue;
        Job& j = s->jobs[it->second];
        s->pass_job.erase(it);
        j.passes_in_flight--;
        j.passes_done++;
        if (j.passes_in_flight > 0) continue;  // a later pass of the job is still coming
        const SceneEntry& sc = s->scenes[j.req.scene_key];
        if (j.req.target_rmse > 0.0 && sc.ref_target >= 0) {
            check.push_back(j.id);
            tgt.push_back(j.target);
            ref.push_back(sc.ref_target);
        } else {
            check.push_back(j.id);
            tgt.push_back(-1);
            ref.push_back(-1);
        }
    }
    // One reduction over every job that has a reference.
    std::vector<int> t2, r2;
    std::vector<size_t> which;
    for (size_t i = 0; i < check.size(); i++)
        if (tgt[i] >= 0) {
            t2.push_back(tgt[i]);
            r2.push_back(ref[i]);
            which.push_back(i);
        }
    std::vector<double> err(t2.size());
    if (!t2.empty()) {
        rc = pt_batch_rmse_many(s->batch, t2.data(), r2.data(), (int)t2.size(), err.data());
        if (rc != PT_OK) return from_batch(s, rc, "rmse");
        for (size_t k = 0; k < which.size(); k++) s->jobs[check[which[k]]].rmse = err[k];
    }
    const double t = now_s(s);
    for (uint64_t id : check) {
        Job& j = s->jobs[id];
        if (done_with(j)) finish(s, j, t);
    }
    s->active.erase(std::remove_if(s->active.begin(), s->active.end(),
                                   [s](uint64_t id) { return s->jobs[id].finished; }),
                    s->active.end());
    return PT_OK;
}

// ---- plain mode ---------------------------------------------------------------

int poll_plain(pt_server* s) {
    if (s->active.empty()) {
        if (s->queue.empty()) return PT_OK;
        Job& j = s->jobs[s->queue.front()];
        s->queue.pop_front();
        j.t_admit = now_s(s);
        s->admitted++;
        s->active.push_back(j.id);
        const SceneEntry& sc = s->scenes[j.req.scene_key];
        if (s->ctx_scene != j.req.scene_key) {
            int rc;
            if (!sc.sources.empty()) {
                std::vector<const char*> src;
                for (const std::string& t : sc.sources) src.push_back(t.c_str());
                rc = pt_set_sdfs(s->ctx, src.data(), (int)src.size());
            } else {
                rc = pt_set_sdf_plugins(s->ctx, sc.plugins.data(), (int)sc.plugins.size());
            }
            if (rc == PT_OK) rc = pt_upload_scene_ext(s->ctx, sc.ubo, sc.ext.get());
            if (rc != PT_OK) return from_ctx(s, rc, "upload");
            s->ctx_scene = j.req.scene_key;
        }
        if (s->ctx_w != j.width || s->ctx_h != j.height) {
            const int rc = pt_resize_accum(s->ctx, j.width, j.height);
            if (rc != PT_OK) return from_ctx(s, rc, "resize");
            s->ctx_w = j.width;
            s->ctx_h = j.height;
        }
    }
    Job& j = s->jobs[s->active.front()];
    const pt_push p = pass_push(j, j.passes_done + 1);
    int rc = pt_dispatch(s->ctx, &p);
    if (rc == PT_OK) rc = pt_wait(s->ctx, UINT64_MAX);
    if (rc != PT_OK) return from_ctx(s, rc, "dispatch");
    j.passes_done++;
    const SceneEntry& sc = s->scenes[j.req.scene_key];
    if (j.req.target_rmse > 0.0 && sc.ref_target >= 0) {
        rc = pt_batch_rmse_image(s->batch, pt_accum_device_ptr(s->ctx), j.width, j.height, sc.ref_target, &j.rmse);
        if (rc != PT_OK) return from_batch(s, rc, "rmse");
    }
    if (done_with(j)) {
        finish(s, j, now_s(s));
        s->active.clear();
    }
    return PT_OK;
}

}  // namespace

extern "C" {

int pt_server_create(pt_server** out, int device, const pt_server_opts* opts) {
    if (!out) return PT_ERR_INVALID;
    *out = nullptr;
    pt_server* s = new (std::nothrow) pt_server();
    if (!s) return PT_ERR_OOM;
    if (opts) s->opts = *opts;
    pt_server_opts& o = s->opts;
    if (o.spp_per_pass <= 0) o.spp_per_pass = 8;
    if (o.hbm_budget == 0) o.hbm_budget = 64ull << 30;
    if (o.pool_slots == 0) o.pool_slots = 1u << 21;
    if (o.max_passes == 0) o.max_passes = 4096;
    if (o.iterations_per_poll <= 0) o.iterations_per_poll = 4;
    if (o.passes_in_flight <= 0) o.passes_in_flight = 1;
    if (o.mode != PT_SERVE_BATCHED && o.mode != PT_SERVE_PLAIN) {
        delete s;
        return PT_ERR_INVALID;
    }
    s->device = device;
    s->t0 = std::chrono::steady_clock::now();
    int rc = pt_batch_create(&s->batch, device, o.pool_slots, o.max_passes);
    if (rc == PT_OK && o.mode == PT_SERVE_PLAIN) {
        rc = pt_create(&s->ctx, device);
        if (rc == PT_OK) rc = pt_set_engine(s->ctx, PT_ENGINE_MEGAKERNEL);
    }
    if (rc != PT_OK) {
        pt_server_destroy(s);
        return rc;
    }
    *out = s;
    return PT_OK;
}

int pt_server_destroy(pt_server* s) {
    if (!s) return PT_ERR_INVALID;
    if (s->ctx) pt_destroy(s->ctx);
    if (s->batch) pt_batch_destroy(s->batch);
    for (auto& kv : s->scenes) delete kv.second.ubo;
    delete s;
    return PT_OK;
}

const char* pt_server_last_error(pt_server* s) { return s ? s->err.c_str() : "null server"; }

int pt_server_set_mode(pt_server* s, int mode) {
    if (!s) return PT_ERR_INVALID;
    if (mode != PT_SERVE_BATCHED && mode != PT_SERVE_PLAIN) return sfail(s, PT_ERR_INVALID, "pt_server_set_mode: mode");
    if (!s->queue.empty() || !s->active.empty() || !s->ready.empty())
        return sfail(s, PT_ERR_BUSY, "pt_server_set_mode: jobs are queued or running");
    if (mode == PT_SERVE_PLAIN && !s->ctx) {
        int rc = pt_create(&s->ctx, s->device);
        if (rc == PT_OK) rc = pt_set_engine(s->ctx, PT_ENGINE_MEGAKERNEL);
        if (rc != PT_OK) return sfail(s, rc, "pt_server_set_mode: context");
        s->ctx_scene = -1;
        s->ctx_w = s->ctx_h = 0;
    }
    s->opts.mode = mode;
    return PT_OK;
}

double pt_server_now(pt_server* s) { return s ? now_s(s) : 0.0; }

pt_batch* pt_server_batch(pt_server* s) { return s ? s->batch : nullptr; }

int pt_server_add_scene(pt_server* s, int key, const pt_ubo* ubo, const pt_sdf_plugin* plugins, int nplugins) {
    if (!s) return PT_ERR_INVALID;
    if (!ubo || nplugins < 0 || (nplugins > 0 && !plugins) || s->scenes.count(key))
        return sfail(s, PT_ERR_INVALID, "pt_server_add_scene: bad arguments or key in use");
    SceneEntry e;
    int rc = pt_batch_add_scene(s->batch, ubo, plugins, nplugins, &e.batch_scene);
    if (rc != PT_OK) return from_batch(s, rc, "pt_server_add_scene");
    e.ubo = new (std::nothrow) pt_ubo;
    if (!e.ubo) return sfail(s, PT_ERR_OOM, "pt_server_add_scene: out of host memory");
    *e.ubo = *ubo;
    e.plugins.assign(plugins, plugins + nplugins);
    s->scenes[key] = std::move(e);
    s->resident_bytes += sizeof(pt_ubo);
    return PT_OK;
}

int pt_server_add_scene_sources(pt_server* s, int key, const pt_ubo* ubo, const char* const* sources, int n) {
    if (!s) return PT_ERR_INVALID;
    if (!ubo || n < 0 || (n > 0 && !sources) || s->scenes.count(key))
        return sfail(s, PT_ERR_INVALID, "pt_server_add_scene_sources: bad arguments or key in use");
    for (int i = 0; i < n; i++)
        if (!sources[i]) return sfail(s, PT_ERR_INVALID, "pt_server_add_scene_sources: null source");
    SceneEntry e;
    int rc = pt_batch_add_scene_sources(s->batch, ubo, sources, n, &e.batch_scene);
    if (rc != PT_OK) return from_batch(s, rc, "pt_server_add_scene_sources");
    e.ubo = new (std::nothrow) pt_ubo;
    if (!e.ubo) return sfail(s, PT_ERR_OOM, "pt_server_add_scene_sources: out of host memory");
    *e.ubo = *ubo;
    e.sources.assign(sources, sources + n);
    s->scenes[key] = std::move(e);
    s->resident_bytes += sizeof(pt_ubo);
    return PT_OK;
}

int pt_server_set_scene_ext(pt_server* s, int key, const pt_scene_ext* ext) {
    if (!s) return PT_ERR_INVALID;
    auto it = s->scenes.find(key);
    if (it == s->scenes.end()) return sfail(s, PT_ERR_INVALID, "pt_server_set_scene_ext: unknown scene key");
    const int rc = pt_batch_set_scene_ext(s->batch, it->second.batch_scene, ext);
    if (rc != PT_OK) return from_batch(s, rc, "pt_server_set_scene_ext");
    it->second.ext = ext ? std::make_shared<pt_scene_ext>(*ext) : nullptr;
    if (s->ctx_scene == key) s->ctx_scene = -1;  // the plain path uploads it again
    return PT_OK;
}

int pt_server_render_reference(pt_server* s, int key, const pt_push* push, int spp, int spp_per_pass) {
    if (!s) return PT_ERR_INVALID;
    auto it = s->scenes.find(key);
    if (it == s->scenes.end() || !push || spp <= 0 || spp_per_pass <= 0 || spp % spp_per_pass != 0)
        return sfail(s, PT_ERR_INVALID, "pt_server_render_reference: bad arguments");
    SceneEntry& e = it->second;
    const int W = push->resolution[0], H = push->resolution[1];
    if (e.ref_target >= 0) {
        pt_batch_release_target(s->batch, e.ref_target);
        s->resident_bytes -= (uint64_t)e.ref_w * (uint64_t)e.ref_h * 32ull;
        e.ref_target = -1;
    }
    int rc = pt_batch_add_target(s->batch, W, H, PT_TARGET_FP64, &e.ref_target);
    if (rc != PT_OK) return from_batch(s, rc, "pt_server_render_reference");
    e.ref_w = W;
    e.ref_h = H;
    s->resident_bytes += (uint64_t)W * (uint64_t)H * 32ull;
    // Sample indices from 2^30 on: independent of every request's samples.
    const bool fp64_paths = s->opts.fp64_paths != 0;
    for (int k = 0; k < spp / spp_per_pass; k++) {
        pt_push p = *push;
        p.samplesPerFrame = spp_per_pass;
        p.frame = (1 << 30) + (k + 1) * spp_per_pass;
        p.currentSamples = spp_per_pass;
        if (fp64_paths) {
            rc = pt_batch_render_fp64(s->batch, e.batch_scene, e.ref_target, &p);
            if (rc != PT_OK) return from_batch(s, rc, "pt_server_render_reference");
            continue;
        }
        int pid = -1;
        rc = pt_batch_add_pass(s->batch, e.batch_scene, e.ref_target, &p, &pid);
        if (rc == PT_ERR_BUSY) {
            rc = pt_batch_run(s->batch, UINT64_MAX);
            if (rc == PT_OK) rc = pt_batch_add_pass(s->batch, e.batch_scene, e.ref_target, &p, &pid);
        }
        if (rc != PT_OK) return from_batch(s, rc, "pt_server_render_reference");
    }
    rc = pt_batch_run(s->batch, UINT64_MAX);
    return from_batch(s, rc, "pt_server_render_reference");
}

int pt_server_submit(pt_server* s, const pt_server_job* req, uint64_t* job_id) {
    if (!s) return PT_ERR_INVALID;
    if (!req || !job_id) return sfail(s, PT_ERR_INVALID, "pt_server_submit: bad arguments");
    auto it = s->scenes.find(req->scene_key);
    if (it == s->scenes.end()) return sfail(s, PT_ERR_INVALID, "pt_server_submit: unknown scene key");
    const int W = req->push.resolution[0], H = req->push.resolution[1];
    if (W <= 0 || H <= 0 || req->push.pathLength <= 0 || req->max_spp <= 0)
        return sfail(s, PT_ERR_INVALID, "pt_server_submit: bad resolution, path length or sample cap");
    if (req->target_rmse > 0.0 && (it->second.ref_target < 0 || it->second.ref_w != W || it->second.ref_h != H))
        return sfail(s, PT_ERR_INVALID, "pt_server_submit: an error target needs the scene's reference at this size");
    Job j;
    j.id = s->next_id++;
    j.req = *req;
    j.width = W;
    j.height = H;
    j.spf = s->opts.spp_per_pass;
    j.t_submit = now_s(s);
    if (s->opts.mode == PT_SERVE_BATCHED && job_bytes(s, j) > s->opts.hbm_budget)
        return sfail(s, PT_ERR_TOO_LARGE, "pt_server_submit: the job alone exceeds the memory budget");
    s->jobs[j.id] = j;
    s->queue.push_back(j.id);
    s->submitted++;
    *job_id = j.id;
    return PT_OK;
}

int pt_server_poll(pt_server* s, pt_server_result* done, int capacity, int* ndone) {
    if (!s) return PT_ERR_INVALID;
    if (!ndone || capacity < 0 || (capacity > 0 && !done)) return sfail(s, PT_ERR_INVALID, "pt_server_poll: bad arguments");
    *ndone = 0;
    const int rc = s->opts.mode == PT_SERVE_BATCHED ? poll_batched(s) : poll_plain(s);
    if (rc != PT_OK) return rc;
    const int n = std::min(capacity, (int)s->ready.size());
    for (int i = 0; i < n; i++) done[i] = s->ready[(size_t)i];
    s->ready.erase(s->ready.begin(), s->ready.begin() + n);
    *ndone = n;
    return PT_OK;
}

int pt_server_pending(pt_server* s) {
    if (!s) return -1;
    return (int)(s->queue.size() + s->active.size() + s->ready.size());
}

int pt_server_cancel(pt_server* s, uint64_t job_id) {
    if (!s) return PT_ERR_INVALID;
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end() || it->second.finished)
        return sfail(s, PT_ERR_INVALID, "pt_server_cancel: unknown or finished job");
    Job& j = it->second;
    j.status = PT_ERR_CANCELLED;
    auto q = std::find(s->queue.begin(), s->queue.end(), job_id);
    if (q != s->queue.end()) {
        s->queue.erase(q);
        finish(s, j, now_s(s));
    } else if (j.passes_in_flight == 0) {  // admitted, between passes (always so on the plain path)
        finish(s, j, now_s(s));
        s->active.erase(std::remove(s->active.begin(), s->active.end(), job_id), s->active.end());
    }  // else it finishes when its passes in flight resolve (poll_batched)
    return PT_OK;
}

int pt_server_read_image(pt_server* s, uint64_t job_id, float* host, size_t bytes) {
    if (!s) return PT_ERR_INVALID;
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end() || !it->second.finished)
        return sfail(s, PT_ERR_INVALID, "pt_server_read_image: unknown or unfinished job");
    const Job& j = it->second;
    if (s->opts.mode == PT_SERVE_PLAIN) {
        if (s->ctx_w != j.width || s->ctx_h != j.height || !s->active.empty())
            return sfail(s, PT_ERR_INVALID, "pt_server_read_image: the plain path keeps only the last job's image");
        return from_ctx(s, pt_read_accum(s->ctx, host, bytes), "pt_server_read_image");
    }
    if (j.target < 0) return sfail(s, PT_ERR_INVALID, "pt_server_read_image: image released (keep_images is off)");
    return from_batch(s, pt_batch_read_target(s->batch, j.target, host, bytes), "pt_server_read_image");
}

int pt_server_release(pt_server* s, uint64_t job_id) {
    if (!s) return PT_ERR_INVALID;
    auto it = s->jobs.find(job_id);
    if (it == s->jobs.end() || !it->second.finished) return sfail(s, PT_ERR_INVALID, "pt_server_release: unknown job");
    if (it->second.target >= 0) pt_batch_release_target(s->batch, it->second.target);
    s->jobs.erase(it);
    return PT_OK;
}

int pt_server_get_stats(pt_server* s, pt_server_stats* out) {
    if (!s || !out) return PT_ERR_INVALID;
    std::memset(out, 0, sizeof *out);
    out->submitted = s->submitted;
    out->admitted = s->admitted;
    out->completed = s->completed;
    out->samples = s->samples;
    out->bytes_in_use = s->bytes_in_use;
    out->bytes_peak = s->bytes_peak;
    out->resident_bytes = s->resident_bytes;
    out->queued = (uint32_t)s->queue.size();
    out->active = (uint32_t)s->active.size();
    return PT_OK;
}

int pt_server_run_trace(pt_server* s, const pt_server_job* reqs, const double* arrivals, int n,
                        pt_server_result* results) {
    if (!s) return PT_ERR_INVALID;
    if (n < 0 || (n > 0 && (!reqs || !arrivals || !results)))
        return sfail(s, PT_ERR_INVALID, "pt_server_run_trace: bad arguments");
    for (int i = 1; i < n; i++)
        if (arrivals[i] < arrivals[i - 1]) return sfail(s, PT_ERR_INVALID, "pt_server_run_trace: unsorted arrivals");
    std::unordered_map<uint64_t, int> index;
    const double start = now_s(s);
    int next = 0, remaining = n;
    std::vector<pt_server_result> buf(256);
    while (remaining > 0) {
        const double t = now_s(s) - start;
        while (next < n && arrivals[next] <= t) {
            uint64_t id = 0;
            const int rc = pt_server_submit(s, &reqs[next], &id);
            if (rc != PT_OK) return rc;
            s->jobs[id].t_submit = start + arrivals[next];  // latency counts from the arrival
            index[id] = next++;
        }
        if (s->queue.empty() && s->active.empty()) {
            if (next < n) {
                const double wait = arrivals[next] - (now_s(s) - start);
                if (wait > 0) std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 0.01)));
            }
            continue;
        }
        int nd = 0;
        const int rc = pt_server_poll(s, buf.data(), (int)buf.size(), &nd);
        if (rc != PT_OK) return rc;
        for (int i = 0; i < nd; i++) {
            pt_server_result r = buf[(size_t)i];
            r.t_submit -= start;
            r.t_admit -= start;
            r.t_done -= start;
            results[index[r.job_id]] = r;
            remaining--;
            if (!s->opts.keep_images) s->jobs.erase(r.job_id);
        }
    }
    return PT_OK;
}

}  // extern "C"
