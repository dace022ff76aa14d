/*
 * pt_host.h — C ABI of libpt_host, the headless host that drives libpt_cuda.
 *
 * It re-states, without GLFW/ImGui/Vulkan, the parts of the reference's
 * src/pathtracer.cpp that sit above the compute dispatch: the scene JSON
 * schema (UpdateFromJSON / UpdateToJSON, :2576-2858), the uniform-buffer
 * packing with its light list (UpdateUniformBuffer, :3642-3811), the push
 * constants (UpdatePushConstant, :3813-3834), the offscreen progressive loop
 * (MainLoop with OFFSCREENRENDER, :3965-4093) and the export tonemap + PPM
 * writer (SaveRender / SavePPM, :3491-3518, :918-933).
 *
 * All calls return PT_OK (0) or a PT_ERR_* code from pt_cuda.h and never
 * throw.  Messages go to the caller's buffer where one is taken.
 */
#ifndef PT_HOST_H
#define PT_HOST_H

#include <stddef.h>
#include <stdint.h>

#include "pt_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct pt_scene pt_scene;

/* Parse a scene JSON document (the reference's schema; "sdf[i].builtin" is
 * accepted in place of "glsl" as "blob" | "mandelbulb" | ... or a full
 * "builtin:<name>[:m0,m1,m2]" spec).  Missing object arrays are empty, as in
 * the reference; missing camera or object fields are errors. */
int pt_scene_parse(const char* json, size_t len, pt_scene** out, char* err, size_t err_cap);
int pt_scene_load_file(const char* path, pt_scene** out, char* err, size_t err_cap);
void pt_scene_free(pt_scene* scene);

/* counts[0..8] = spheres, planes, boxes, lenses, cyclides, sdfs, materials,
 * lights, camera shots. */
int pt_scene_counts(const pt_scene* scene, int counts[9]);

/* UpdateUniformBuffer: pack objects, SDF boxes, materials, lights and the
 * light-ID list (with the reference's lens/cyclide light-list quirk), and
 * copy `cie` (1323 floats) into the table.  Fails with PT_ERR_INVALID when
 * the scene overflows the fixed arrays (the reference truncates silently). */
int pt_scene_pack_ubo(const pt_scene* scene, const float* cie, pt_ubo* out);

/* The scene's full-form extensions (include/pt_cuda.h, pt_scene_ext) from
 * the JSON keys the reference's loader ignores: "environment"
 * {temperature, luminosity} (a blackbody sky), "spectral" {range: [min, max]
 * nm, cmf: "analytic" | "table"}, "march" {maxSteps, epsilon, maxDistance}
 * and per material "bsdf" {type: "flat" albedo | "smooth" base, amplitude,
 * center, width | "mirror" reflectance | "cauchy" A, B | "sellmeier" B[3],
 * C[3]}.  A scene without them gives flags == 0.  pt_scene_bind uploads
 * them with the scene. */
int pt_scene_pack_ext(const pt_scene* scene, pt_scene_ext* out);

/* The host's progressive-render state that UpdatePushConstant reads. */
typedef struct pt_frame_state {
    int32_t width, height;
    int32_t frame;           /* samples issued so far including this dispatch */
    int32_t currentSamples;  /* samples in the running mean after this dispatch */
    int32_t samplesPerFrame;
    float FPS;               /* 1 / frameTime */
    float persistence;       /* reference default 0.0625 */
    int32_t pathLength;
    int32_t cameraShotIndex; /* 1-based, reference default 1 */
    int32_t tonemap;         /* 0 none, 1 Reinhard, 2 ACES, 3 DEUCES (reference default 3) */
} pt_frame_state;

/* UpdatePushConstant. */
int pt_scene_push_constants(const pt_scene* scene, const pt_frame_state* st, pt_push* out);

/* Source text of SDF i (its "glsl", or the builtin spec), owned by the scene. */
const char* pt_scene_sdf_source(const pt_scene* scene, int i);

/* UpdateToJSON + dump(4): writes a NUL-terminated document of at most cap
 * bytes; *needed receives the full size including the NUL. */
int pt_scene_to_json(const pt_scene* scene, char* buf, size_t cap, size_t* needed);

/* Pack + pt_set_sdfs + pt_upload_scene on a context (a scene load and the
 * recompile it triggers in the reference, :3442-3461 and :3836-3841). */
int pt_scene_bind(pt_ctx* ctx, const pt_scene* scene, const float* cie);

/* The scene's SDF plug-ins (each SDF's source through pt_parse_sdf_source),
 * for pt_batch_add_scene: writes min(count, cap) entries, *count = SDFs. */
int pt_scene_sdf_plugins(const pt_scene* scene, pt_sdf_plugin* out, int cap, int* count);

/* Seeded synthetic render jobs.  No counterpart in the reference: stand-ins
 * for a stream of user scenes, deterministic per seed on every platform
 * (std::mt19937_64 plus libm-free transforms), expressed in the reference's
 * scene schema and method.
 *   PT_GEN_SPHERES  4-64 spheres, centres U[-2,2]^3, radii lognormal(-1.5,
 *                   0.5), three material classes, on a ground plane, one
 *                   blackbody sphere light at 3000-9000 K; W = H uniform over
 *                   {128, 256, 512, 1024}; spp log-uniform over [4, 256];
 *                   path length 8.
 *   PT_GEN_SDF      a mandelbulb, menger or blob plug-in over a ground plane
 *                   under a sky and a sun; W = H uniform over {256, 512,
 *                   1024}; spp 0 (open); path length 8.
 *   PT_GEN_SDF_VARIED  the same scenes with the mandelbulb's power uniform
 *                   over [4, 10] (4-6 iterations) and the menger's levels
 *                   uniform over {3, 4, 5}, given as GLSL text (compiled at
 *                   run time: pt_set_sdfs, pt_batch_add_scene_sources). */
#define PT_GEN_SPHERES 0
#define PT_GEN_SDF 1
#define PT_GEN_SDF_VARIED 2
#define PT_GEN_SPHERES_FULL 3 /* PT_GEN_SPHERES' scenes with mirror and Cauchy dielectric models (extension "bsdf") */
typedef struct pt_job_spec {
    int32_t kind;
    int32_t width, height;
    int32_t spp;
    int32_t pathLength;
    int32_t sdf_kind; /* PT_SDF_* of an SDF job, PT_SDF_NONE otherwise */
    int32_t objects;  /* spheres of a sphere job (light excluded), 1 for an SDF job */
    int32_t pad;
    uint64_t seed;
} pt_job_spec;
int pt_scene_generate(int kind, uint64_t seed, pt_scene** out, pt_job_spec* spec);

/* The reference's offscreen render (numSamples, samplesPerFrame, path length
 * and shot index read from stdin there): frame += spf per dispatch until
 * currentSamples >= numSamples, then the accumulator is read back. */
typedef struct pt_offscreen_opts {
    int32_t width, height;
    int32_t numSamples;
    int32_t samplesPerFrame;
    int32_t pathLength;
    int32_t cameraShotIndex;
    int32_t tonemap;
    int32_t frameOffset; /* samples already issued before this render (0 in the reference) */
} pt_offscreen_opts;
int pt_render_offscreen(pt_ctx* ctx, const pt_scene* scene, const float* cie, const pt_offscreen_opts* opts,
                        float* accum_out, size_t accum_bytes, double* seconds_out);

/* SaveRender's per-pixel chain: E->D65 Bradford, XYZ->sRGB, max(0), tonemap,
 * sRGB companding, 8-bit truncation.  rgb_out holds W*H*3 bytes. */
int pt_export_rgb8(const float* accum, int width, int height, int tonemap, uint8_t* rgb_out);
/* SavePPM: binary P6 with "P6\nW\nH\n255\n" header. */
int pt_save_ppm(const char* path, const uint8_t* rgb, int width, int height);

/* CIE 1931 2-degree colour-matching functions at 1 nm over 360..800 nm from
 * the multi-lobe Gaussian fit of Wyman, Sloan & Shirley (JCGT 2(2), 2013),
 * x y z interleaved: a caller-supplied table for pt_ubo.CIEXYZ1931. */
void pt_cie_analytic_table(float out[PT_CIE_TABLE_SIZE]);

/* ---------------------------------------------------------------------------
 * Render serving.  No counterpart in the reference, whose host renders one
 * scene at a time: requests name a resident scene and a target error; each
 * admitted job is refined with progressive passes of spp_per_pass samples
 * (pass k: frame = currentSamples = k * spp_per_pass, the reference's
 * offscreen loop) until its relative RMSE (pt_batch_rmse) against the scene's
 * FP64 reference is at most target_rmse, or max_spp is reached.
 *   PT_SERVE_BATCHED  continuous batching on a pt_batch: requests are
 *                     admitted in arrival order while their accumulator and
 *                     in-flight sample colours fit hbm_budget; the passes of
 *                     all admitted jobs share every launch.
 *   PT_SERVE_PLAIN    one job at a time through pt_dispatch on the plain
 *                     megakernel (the drop-in path), for comparison.
 * A job's image after k passes is the same bits in both modes, alone or in
 * any mix.  Times are seconds on the server's monotonic clock.
 * ------------------------------------------------------------------------- */
typedef struct pt_server pt_server;

#define PT_SERVE_BATCHED 0
#define PT_SERVE_PLAIN 1

typedef struct pt_server_opts {
    int32_t mode;                /* PT_SERVE_* */
    int32_t spp_per_pass;        /* default 8 */
    uint64_t hbm_budget;         /* bytes for admitted jobs (default 64 GiB) */
    uint32_t pool_slots;         /* staged-engine path slots (default 2^21) */
    uint32_t max_passes;         /* passes in flight per engine (default 4096) */
    int32_t iterations_per_poll; /* engine iterations per pt_server_poll (default 4) */
    int32_t passes_in_flight;    /* per job (default 1) */
    int32_t keep_images;         /* keep finished images until pt_server_release */
    int32_t fp64_paths;          /* references traced in double precision (pt_batch_render_fp64) instead of
                                    FP32 paths summed in double (the default, 0) */
} pt_server_opts;

typedef struct pt_server_job {
    int32_t scene_key;
    int32_t max_spp;     /* sample cap per pixel */
    double target_rmse;  /* stop at this relative RMSE vs the reference (0: run to max_spp) */
    pt_push push;        /* resolution, camera, pathLength; frame/currentSamples/samplesPerFrame set per pass */
} pt_server_job;

typedef struct pt_server_result {
    uint64_t job_id;
    int32_t status;
    int32_t spp;       /* samples per pixel rendered */
    double rmse;       /* at completion; -1 without a reference */
    double t_submit;   /* arrival */
    double t_admit;
    double t_done;     /* time to target = t_done - t_submit */
    uint64_t samples;  /* path samples rendered for the job */
} pt_server_result;

typedef struct pt_server_stats {
    uint64_t submitted, admitted, completed;
    uint64_t samples;
    uint64_t bytes_in_use, bytes_peak; /* admitted jobs, against hbm_budget */
    uint64_t resident_bytes;           /* FP64 references and scene copies */
    uint32_t queued, active;
} pt_server_stats;

int pt_server_create(pt_server** out, int device, const pt_server_opts* opts);
int pt_server_destroy(pt_server* server);
const char* pt_server_last_error(pt_server* server);
double pt_server_now(pt_server* server);
/* Switches between PT_SERVE_BATCHED and PT_SERVE_PLAIN while no job is
 * queued or running; scenes and references stay resident. */
int pt_server_set_mode(pt_server* server, int mode);
/* The batch the server renders with (scenes, references, statistics). */
pt_batch* pt_server_batch(pt_server* server);
/* Makes a scene resident under `key`. */
int pt_server_add_scene(pt_server* server, int key, const pt_ubo* ubo, const pt_sdf_plugin* plugins, int nplugins);
/* Makes a scene resident whose SDFs are given as text (pt_batch_add_scene_sources;
 * the plain path sets them with pt_set_sdfs). */
int pt_server_add_scene_sources(pt_server* server, int key, const pt_ubo* ubo, const char* const* sources, int n);
/* Full-form extensions of a resident scene (NULL: the reference's method),
 * for both modes; PT_ERR_BUSY while jobs of the scene are in flight. */
int pt_server_set_scene_ext(pt_server* server, int key, const pt_scene_ext* ext);
/* Renders scene `key`'s FP64 reference for a view (push: resolution, camera,
 * path length) with spp samples per pixel from sample indices no request
 * uses; blocks until done.  With opts.fp64_paths the paths themselves are
 * traced in double precision (pt_batch_render_fp64). */
int pt_server_render_reference(pt_server* server, int key, const pt_push* push, int spp, int spp_per_pass);
int pt_server_submit(pt_server* server, const pt_server_job* job, uint64_t* job_id);
/* Admits, feeds and advances the work once; returns jobs finished since the
 * last call (up to capacity; the rest on later calls). */
int pt_server_poll(pt_server* server, pt_server_result* done, int capacity, int* ndone);
/* Jobs queued, active or finished but not yet returned by pt_server_poll. */
int pt_server_pending(pt_server* server);
/* Cancels a job that has not finished: a queued job is dropped at once; an
 * admitted one gets no further passes and finishes when its passes in flight
 * have resolved.  pt_server_poll then returns it with status
 * PT_ERR_CANCELLED and the samples it rendered. */
int pt_server_cancel(pt_server* server, uint64_t job_id);
int pt_server_read_image(pt_server* server, uint64_t job_id, float* host, size_t bytes);
int pt_server_release(pt_server* server, uint64_t job_id);
int pt_server_get_stats(pt_server* server, pt_server_stats* out);
/* Replays an arrival trace: request i is submitted `arrivals[i]` seconds
 * (non-decreasing) after the call and results[i] receives its outcome, with
 * times relative to the call.  Returns when every request has finished. */
int pt_server_run_trace(pt_server* server, const pt_server_job* jobs, const double* arrivals, int n,
                        pt_server_result* results);

#ifdef __cplusplus
}
#endif

#endif /* PT_HOST_H */
