/*
 * pt_cuda.h — C ABI of libpt_cuda, the GB300 (sm_103a) replacement for the
 * Vulkan compute dispatch of phyastro/PathTracer.
 *
 * The reference host packs a scene into a float uniform buffer, pushes 88 bytes
 * of push constants, dispatches src/shader.comp over ceil(W/16) x ceil(H/16)
 * workgroups and waits on a fence; the shader read-modify-writes an RGBA32F
 * texel buffer holding the running mean of CIE XYZ per pixel.  This library
 * exposes the same contract as plain C calls: the byte layouts of pt_ubo and
 * pt_push are identical to the reference's UniformBufferObject and
 * PushConstantValues, and the accumulator has the reference's layout
 * (float4 XYZ + w=1 at index x + W*y over invocation coordinates).
 *
 * Conventions
 *   - Every call returns a status code (PT_OK == 0); no exception crosses the
 *     ABI.  pt_last_error() returns a message for the last failing call.
 *   - The context owns all device memory.  Input structs are copied at call
 *     time; the caller keeps ownership of its buffers.
 *   - A context is single-threaded (one stream, like the reference's one
 *     compute queue); distinct contexts may be used from distinct threads.
 */
#ifndef PT_CUDA_H
#define PT_CUDA_H

#if !defined(__CUDACC_RTC__)
#include <stddef.h>
#include <stdint.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Sizes of the uniform-buffer arrays (src/pathtracer.cpp:39-43, src/shader.comp:11-15). */
#define PT_MAX_OBJECTS_SIZE 1024
#define PT_MAX_SDFS_SIZE 768
#define PT_MAX_MATERIALS_SIZE 783
#define PT_MAX_LIGHTS_SIZE 128
#define PT_MAX_LIGHTIDS_SIZE 64
#define PT_CIE_TABLE_SIZE 1323 /* 441 wavelengths 360..800 nm, x y z interleaved */
/* SDF slots that the shader can evaluate: SearchSDF builds a 32-bit set mask
 * and set2..set4 are never filled (src/shader.comp:732-777). */
#define PT_MAX_LIVE_SDFS 32

/* Status codes. */
#define PT_OK 0
#define PT_ERR_INVALID 1       /* bad argument (null pointer, size, layout) */
#define PT_ERR_CUDA 2          /* a CUDA runtime call failed */
#define PT_ERR_TIMEOUT 3       /* pt_wait deadline passed; the work is still queued */
#define PT_ERR_UNSUPPORTED 4   /* e.g. an SDF plug-in source that is not recognised */
#define PT_ERR_NO_SCENE 5      /* dispatch before pt_upload_scene / pt_resize_accum */
#define PT_ERR_OOM 6           /* device allocation failed */
#define PT_ERR_KERNEL 7        /* the device work did not complete within its iteration limit (wavefront drain,
                                  batch run), or an index check of the checked kernel build failed */
#define PT_ERR_TOO_LARGE 8     /* the request exceeds pt_dispatch_noalloc's fixed scratch */
#define PT_ERR_BUSY 9          /* the resource is still in use by passes in flight */
#define PT_ERR_CANCELLED 10    /* a served job was cancelled (pt_server_cancel) */

/* Byte-for-byte the reference's UniformBufferObject (src/pathtracer.cpp:187-195)
 * and the shader's `ubo` block (src/shader.comp:19-27): 4097 floats = 16388 B.
 * Object/material/light IDs are stored as floats, 1-based, 0 = none. */
typedef struct pt_ubo {
    float numObjects[7]; /* spheres, planes, boxes, lenses, cyclides, sdfs, lights */
    float objects[PT_MAX_OBJECTS_SIZE];
    float sdfs[PT_MAX_SDFS_SIZE];
    float materials[PT_MAX_MATERIALS_SIZE];
    float lights[PT_MAX_LIGHTS_SIZE];
    float lightIDs[PT_MAX_LIGHTIDS_SIZE];
    float CIEXYZ1931[PT_CIE_TABLE_SIZE];
} pt_ubo;

/* Byte-for-byte the reference's PushConstantValues (src/pathtracer.cpp:197-218)
 * and the shader's push-constant block (src/shader.comp:31-52): 88 B. */
typedef struct pt_push {
    int32_t resolution[2];
    int32_t frame;          /* samples issued so far, including this dispatch */
    int32_t currentSamples; /* samples in the running mean after this dispatch */
    int32_t samplesPerFrame;
    float FPS;
    float persistence;
    int32_t pathLength;
    float cameraAngle[2]; /* (-angle.y, angle.x) in degrees, as the host pushes it */
    float cameraPosX;
    float cameraPosY;
    float cameraPosZ;
    int32_t ISO;
    float cameraSize;
    float apertureSize;
    float apertureDist;
    float lensRadius;
    float lensFocalLength;
    float lensThickness;
    float lensDistance;
    int32_t tonemap;
} pt_push;

/* SDF plug-ins.  The reference splices GLSL snippets defining
 * `float sdf(in vec3 p)` / `float sdfmaterial(in vec3 p)` into the shader
 * (src/pathtracer.cpp:2004-2054).  The four shipped snippets (sdfs/<name>.glsl)
 * are CUDA __device__ functions here; `material` carries the constants that
 * the scene files vary in their copies of sdfmaterial. */
enum {
    PT_SDF_NONE = 0,
    PT_SDF_BLOB = 1,       /* sdfs/blob.glsl: material = lobe IDs (default 4,5,6) */
    PT_SDF_MANDELBULB = 2, /* sdfs/mandelbulb.glsl: material = mix endpoints (default 4,3) */
    PT_SDF_MENGER = 3,     /* sdfs/menger.glsl: material[0] constant (default 0) */
    PT_SDF_TERRAIN = 4,    /* sdfs/terrain.glsl: material[0] constant (default 0) */
    PT_SDF_CUSTOM = 5      /* other GLSL text: compiled at run time (pt_set_sdfs only) */
};
enum {
    PT_SDFMAT_DEFAULT = 0,  /* the snippet's own sdfmaterial form with `material` */
    PT_SDFMAT_CONSTANT = 1  /* sdfmaterial returns material[0] */
};
typedef struct pt_sdf_plugin {
    int32_t kind;
    int32_t material_mode;
    float material[3];
} pt_sdf_plugin;

typedef struct pt_ctx pt_ctx;

/* Create a context on CUDA device `device` (replaces instance/device/pipeline
 * creation, src/pathtracer.cpp:1227-2092). */
int pt_create(pt_ctx** out, int device);
int pt_destroy(pt_ctx* ctx);

/* Replaces InsertSDF + GLSLToSPIRV + RecompileComputeShaders
 * (src/pathtracer.cpp:2004-2054, 1811-1868, 3836-3841).  Each source is the
 * GLSL text of a scene's `sdf[i].glsl` or a spec
 * "builtin:<blob|mandelbulb|menger|terrain>[:m0,m1,m2]".  The reference's
 * four snippets (recognised by a whitespace-insensitive fingerprint) map to
 * precompiled plug-ins; any other text is translated (pt_glsl_translate) and
 * compiled at run time, on the first dispatch of each engine (seconds, then
 * cached), into the megakernel or the wavefront engine's march kernel.
 * Positions and bounding boxes come from pt_ubo.sdfs, as in the reference. */
int pt_set_sdfs(pt_ctx* ctx, const char* const* sources, int n);
/* Same, from already-decoded descriptors. */
int pt_set_sdf_plugins(pt_ctx* ctx, const pt_sdf_plugin* plugins, int n);
/* Decode one source string into a descriptor without a context. */
int pt_parse_sdf_source(const char* source, pt_sdf_plugin* out);
/* The whitespace-insensitive FNV-1a-64 fingerprint pt_parse_sdf_source
 * matches GLSL text by (0 for NULL). */
uint64_t pt_sdf_source_fingerprint(const char* source);

/* GLSL SDF snippet (a scene's `sdf[i].glsl`: `float sdf(in vec3 p)` and
 * `float sdfmaterial(in vec3 p)` plus helpers) to C++ over the GLSL shim the
 * run-time compiled kernels include, every function renamed <prefix><name>
 * and the text wrapped in namespace ptg::<prefix> (prefix: an identifier).
 * Writes a NUL-terminated text of at most cap bytes (*needed: its size);
 * PT_ERR_UNSUPPORTED with a reason in err for what the shim does not cover. */
int pt_glsl_translate(const char* glsl, const char* prefix, char* out, size_t cap, size_t* needed, char* err,
                      size_t err_cap);
/* Compiles (without loading) the run-time kernels a context builds for n
 * snippets (megakernel, march kernel, FP64 renderer) for compute capability
 * sm (e.g. 103): a check that needs no GPU.  The log receives the
 * compiler's messages. */
int pt_jit_check(const char* const* sources, int n, int sm, char* log, size_t log_cap);

/* Replaces the UBO upload (src/pathtracer.cpp:3805-3807). */
int pt_upload_scene(pt_ctx* ctx, const pt_ubo* ubo);

/* ---- full-form scene extensions (not in the reference) ------------------
 * The reference shades every surface with one Lambertian BRDF whose
 * reflectance is a Gaussian bump (src/shader.comp:1030-1038, :1075-1091), a
 * ray that leaves the scene returns nothing (:1383-1389), hero wavelengths
 * rotate through [390, 720) nm with the tabulated CIE table (:960-974,
 * :129-140) and sphere tracing runs up to 512 steps with no distance cap
 * (:779-860).  A pt_scene_ext adds, per scene and only where its flag is
 * set: an environment sky (blackbody, PT_EXT_SKY), a wavelength range other
 * than the reference's (PT_EXT_WAVELENGTHS), the analytic multi-lobe CIE fit
 * evaluated per wavelength instead of the table (PT_EXT_ANALYTIC_CMF), march
 * limits (PT_EXT_MARCH), and other surface models for materials 1..nmat
 * (PT_EXT_MATERIALS).  A zeroed pt_scene_ext is the reference's method,
 * bit for bit; the scene JSON carries the same fields under keys the
 * reference's loader ignores. */
enum {
    PT_EXT_SKY = 1,
    PT_EXT_WAVELENGTHS = 2,
    PT_EXT_ANALYTIC_CMF = 4,
    PT_EXT_MARCH = 8,
    PT_EXT_MATERIALS = 16
};
enum {
    PT_BSDF_REFERENCE = 0, /* the reference's Lambertian with its Gaussian-bump reflectance */
    PT_BSDF_FLAT = 1,      /* Lambertian, reflectance p[0] at every wavelength */
    PT_BSDF_SMOOTH = 2,    /* Lambertian, reflectance p[0] + p[1] exp(-((l - p[2]) / p[3])^2), l in nm */
    PT_BSDF_MIRROR = 3,    /* conductor mirror: specular reflection, reflectance p[0] */
    PT_BSDF_CAUCHY = 4,    /* dielectric, n(l) = p[0] + p[1] / l^2 (l in um) */
    PT_BSDF_SELLMEIER = 5  /* dielectric, n(l)^2 = 1 + sum_i p[i] l^2 / (l^2 - p[3+i]) (l in um, C in um^2) */
};
#define PT_MAX_EXT_MATERIALS 128
typedef struct pt_material_ext {
    int32_t type; /* PT_BSDF_* */
    float p[6];
} pt_material_ext;
typedef struct pt_scene_ext {
    int32_t flags;            /* PT_EXT_* */
    float sky_temperature;    /* K: the sky's emission is Emit's normalised Planck spectrum x luminosity */
    float sky_luminosity;
    float lambda_min;         /* nm: hero and rotated wavelengths uniform over [lambda_min, lambda_max) */
    float lambda_max;
    int32_t march_max_steps;  /* sphere-tracing steps (the reference: 512); exhausting them counts as a hit */
    float march_epsilon;      /* hit when |d| < epsilon (the reference: 1e-4) */
    float march_max_distance; /* a march past this ray distance misses (the reference: none) */
    int32_t nmat;             /* materials 1..nmat have an entry below (<= PT_MAX_EXT_MATERIALS) */
    pt_material_ext mat[PT_MAX_EXT_MATERIALS];
} pt_scene_ext;
/* pt_upload_scene with extensions (NULL: the reference's method). */
int pt_upload_scene_ext(pt_ctx* ctx, const pt_ubo* ubo, const pt_scene_ext* ext);

/* Replaces CreateTexelBuffer (src/pathtracer.cpp:2250-2256): a zeroed
 * W*H float4 accumulator (at the current size: the same buffer, zeroed in
 * stream order; another size: a new buffer, after the stream drains). */
int pt_resize_accum(pt_ctx* ctx, int width, int height);

/* Replaces RecordComputeCommandBuffer + vkQueueSubmit
 * (src/pathtracer.cpp:3586-3608, 3843-3880).  Asynchronous on the context's
 * stream; resolution must equal the accumulator size. */
int pt_dispatch(pt_ctx* ctx, const pt_push* push);

/* The FP64 reference renderer (no counterpart in the reference): the
 * dispatch's paths (push: resolution, samples, path length, camera) traced
 * with the same method in double precision, each pixel's exposed colour
 * sum (Rendering's apertureSize^2 * ISO, src/shader.comp:1517) and sample
 * count added to d_sums (W*H*4 doubles, device memory, zeroed by the
 * caller before the first call; mean = sum / count).  It draws the same
 * random stream as pt_dispatch for the same push constants, so the two
 * images differ only by the FP32 arithmetic's error and the few paths whose
 * branches it changes.  SDF text compiled at run time is compiled once more
 * for it, with every GLSL float a double (the text's literals keep their
 * float values).  Asynchronous on the context's stream (pt_wait);
 * pt_set_trace applies. */
int pt_render_fp64(pt_ctx* ctx, const pt_push* push, double* d_sums);

/* Engines behind pt_dispatch; both compute the reference's per-sample
 * arithmetic bit for bit and differ only in scheduling.
 *   PT_ENGINE_MEGAKERNEL: one thread per pixel, samples in order (the plain
 *     method).  Asynchronous.
 *   PT_ENGINE_WAVEFRONT (default): every sample is a work item in a pool of
 *     path slots in device memory; compacted ray queues per stage and a
 *     persistent SDF-march kernel; per-sample XYZ summed per pixel in sample
 *     order at the end.  Allocates its scratch on first use; pt_dispatch
 *     returns once the dispatch is resolved on the stream. */
#define PT_ENGINE_MEGAKERNEL 0
#define PT_ENGINE_WAVEFRONT 1
int pt_set_engine(pt_ctx* ctx, int engine);
int pt_get_engine(pt_ctx* ctx);
/* Path slots of the wavefront pool (default 2^22: a deeper pool keeps more
 * rays to refill march lanes from; 252 B each, plus 16 B per sample of the
 * dispatch for the sample colours; a dispatch uses at most its own sample
 * count of slots). */
int pt_set_wavefront_pool(pt_ctx* ctx, uint32_t slots);
/* Wavefront engines a large dispatch is split between (1..4; default 2).
 * A dispatch of at least two pools' worth of samples per engine is rendered
 * by up to that many engines with a pool each, on streams of their own (the
 * context's stream and streams the context owns, forked from and joined
 * back to it), each taking an equal share of the dispatch's samples in
 * sample order: one engine's kernels fill the SMs that the others' kernel
 * tails and host round trips leave idle.  The same bits as one engine
 * (every sample's colour lands in the dispatch's colour buffer and is
 * summed per pixel in sample order).  Each engine holds a pool (lowering
 * the count frees the pools past it); one engine runs when a trace or stage
 * timing is on. */
int pt_set_wavefront_engines(pt_ctx* ctx, int engines);
int pt_get_wavefront_engines(pt_ctx* ctx);
/* Sphere-tracing iterations a ray may take per march launch before it is
 * suspended to the next wavefront iteration (default 64, 1..512). */
int pt_set_march_budget(pt_ctx* ctx, int steps);
/* Wavefront iterations the last dispatch needed (diagnostics; split between
 * two engines: the larger engine's count). */
uint32_t pt_last_iterations(pt_ctx* ctx);
/* Kernels the last pt_dispatch launched (diagnostics; a wavefront dispatch
 * counts each iteration's stage kernels, pass setup and the resolve). */
uint64_t pt_last_kernel_launches(pt_ctx* ctx);

/* Replaces vkWaitForFences (src/pathtracer.cpp:3846): waits at most
 * timeout_ns and returns PT_ERR_TIMEOUT instead of blocking forever. */
int pt_wait(pt_ctx* ctx, uint64_t timeout_ns);

/* Replaces the mapped read of the texel buffer in SaveRender
 * (src/pathtracer.cpp:3496-3515).  Synchronous.  bytes >= W*H*16. */
int pt_read_accum(pt_ctx* ctx, float* host, size_t bytes);
/* Uploads a host accumulator (resume a progressive render).  Synchronous. */
int pt_write_accum(pt_ctx* ctx, const float* host, size_t bytes);
/* SaveRender's tonemap chain (src/pathtracer.cpp:3491-3518: E->D65,
 * XYZ->sRGB, max(0), tonemap 0-3, sRGB companding, byte truncation) on the
 * device.  No reference counterpart as a device call; the same bytes as
 * pt_export_rgb8 in libpt_host.
 *   pt_export_rgb8_device: caller's W*H float4 -> W*H*3 bytes, asynchronous
 *     on `stream` (a cudaStream_t, NULL for the default stream);
 *   pt_read_rgb8: the context's accumulator into a host buffer of W*H*3
 *     bytes (3 bytes per pixel cross the bus instead of 16). */
int pt_export_rgb8_device(const void* d_accum, int width, int height, int tonemap, void* d_rgb, void* stream);
int pt_read_rgb8(pt_ctx* ctx, int tonemap, uint8_t* host_rgb, size_t bytes);

/* Device address of the accumulator (float4 per pixel), or NULL. */
void* pt_accum_device_ptr(pt_ctx* ctx);

/* The cudaStream_t the context launches on (as void*), and a way to replace
 * it with a caller-owned stream (NULL restores the context's own stream).
 * A replaced stream must outlive every later call on the context, pt_destroy
 * included (it synchronises the stream): restore NULL before the stream's
 * owner — possibly another context — destroys it. */
void* pt_stream(pt_ctx* ctx);
int pt_set_stream(pt_ctx* ctx, void* stream);

/* Message of the last failing call on this context (never NULL). */
const char* pt_last_error(pt_ctx* ctx);

/* ---- verification hooks (not in the reference) --------------------------
 * Per-path branch trace of the next dispatch: for every invocation (x, y)
 * and sample k, path index p = (y * W + x) * samplesPerFrame + k; events
 * [p * depth_cap + i] holds bounce i's event word (PT_EV_* below), nevents[p]
 * the number of bounces, colors[p*3..] the sample's XYZ before averaging.
 * Device pointers owned by the caller; pass NULLs to disable. */
int pt_set_trace(pt_ctx* ctx, uint32_t* d_events, uint32_t* d_nevents, float* d_colors, int depth_cap);

/* FMA contraction for the kernels this context compiles at run time (scene
 * GLSL beyond the shipped snippets: the megakernel, or the wavefront engine's
 * march kernel), from their next compilation on (no counterpart in the
 * reference).  Off (the default): every a*b+c rounds twice, as the shader's
 * expressions are written, and results are the reference's bit for bit.  On:
 * the compiler may fuse a*b+c into one fma — fewer instructions in the
 * issue-bound march, results within FP32 rounding of the method, no longer
 * bit-identical. */
int pt_set_fp_contract(pt_ctx* ctx, int on);

/* The wavefront engine's kernels built with index checks (no counterpart
 * in the reference; a substitute for a device memory checker): every queue
 * append, slot read from a queue or the free list, pass index and sample
 * index is checked before use.  A failed check skips its access and makes
 * the dispatch return PT_ERR_KERNEL, naming the site and the index, with
 * the accumulator unchanged.  With every check passing, results are the
 * unchecked kernels' bit for bit.  Off by default (the checks cost time);
 * run-time compiled march kernels are compiled again for the checked build.
 * The plain megakernel has no queues and is not affected. */
int pt_set_device_checks(pt_ctx* ctx, int on);

/* Caps the iterations of the next wavefront dispatches' drain (0: the bound
 * the library computes from the dispatch's size, path length and march
 * budget, which a correct dispatch never reaches).  A dispatch that reaches
 * the cap returns PT_ERR_KERNEL with its accumulator unchanged; the context
 * stays usable.  For tests of that limit. */
int pt_set_drain_limit(pt_ctx* ctx, uint64_t max_iterations);

/* Evaluates one include/pt_mathf.h function on the device over device
 * arrays (fn 0 sin, 1 cos, 2 exp, 3 log, 4 pow(x, y), 5 acos, 6 asin,
 * 7 atan, 8 atan2(x, y) (GLSL atan(y, x) with y the first array), 9 exp2,
 * 10 log2), so tests can compare its bits with the same function on the
 * CPU.  Synchronous. */
int pt_mathf_eval(pt_ctx* ctx, int fn, const float* d_x, const float* d_y, float* d_out, int n);

/* Evaluates the two quartic surfaces the reference's shader defines but
 * never calls (Thritorius, src/shader.comp:543-588, which 0; SmoothCuboid,
 * :590-631, which 1; their call sites :926-931 and :1207-1216 are commented
 * out, so no scene reaches them) for n rays: d_rays6 origin + direction per
 * ray, d_hits6 the hit record (hitdist, normal, materialID, lightID) read and
 * updated as the shader's inout arguments, d_flags the boolean result.
 * Device arrays; synchronous.  For tests against the CPU restatement. */
int pt_quartic_surface_eval(pt_ctx* ctx, int which, const float* d_rays6, float* d_hits6, int* d_flags, int n);

/* ---- dispatch without allocating (not in the reference) -----------------
 * No counterpart in the reference.  One wavefront dispatch (the engine
 * PT_ENGINE_WAVEFRONT runs, bit-identical results) for callers that cannot
 * allocate device memory while they render: a plug-in whose host application
 * owns the GPU memory budget and forbids allocations after start-up, or a
 * real-time loop that cannot pay an allocator's latency or fragmentation.
 * The caller passes the scene and push constants in host memory and the
 * accumulator (W*H float4, read and written as by pt_dispatch) in its own
 * device memory; all working memory of the call lives in one fixed array of
 * PT_NOALLOC_SCRATCH_BYTES (32 MiB) in the library's device image, which
 * every GPU that loads the library holds until the process exits.
 * Limits: W*H*samplesPerFrame <= PT_NOALLOC_MAX_SAMPLES per call (else
 * PT_ERR_TOO_LARGE), PT_NOALLOC_POOL_SLOTS path slots, devices 0..63, the
 * shipped SDF plug-ins only (PT_SDF_CUSTOM: PT_ERR_UNSUPPORTED).
 * The first call on each device looks up the array's device address; with
 * lazy module loading (the CUDA default) that first call also commits the
 * array's 32 MiB, so make it once as a warm-up: later calls allocate
 * nothing.  All calls share the array, so calls that
 * overlap on the GPU race; the counters are reset at the start of every
 * call.  A per-device host lock is held for the whole call and the call
 * returns only when the dispatch is complete on `stream` (NULL: the default
 * stream), so calls from several host threads run one after another.  No
 * per-path trace. */
#define PT_NOALLOC_SCRATCH_BYTES (32u << 20)
#define PT_NOALLOC_MAX_SAMPLES (1u << 20)
#define PT_NOALLOC_POOL_SLOTS (15u << 12) /* 61,440 */
int pt_dispatch_noalloc(const pt_ubo* ubo, const pt_sdf_plugin* plugins, int nplugins, const pt_push* push,
                        float* d_accum, void* stream);

/* Knobs of the wavefront engine (no counterpart in the reference).  The
 * defaults suit the SDF scenes measured on GB300; pt_autotune_wavefront
 * picks them for a given scene and dispatch shape. */
typedef struct pt_wavefront_tuning {
    uint32_t pool_slots;   /* path slots (1024..2^28; default 2^22) */
    int32_t march_budget;  /* SDF steps per ray per march launch (1..512; default 64) */
    int32_t refill_min;    /* idle lanes a march warp gathers before refilling them together (1..32) */
    int32_t drain_lanes;   /* a march warp left with fewer rays after its queue drained suspends them (0..32) */
    int32_t blocks_per_sm; /* stage-kernel blocks of 256 threads per SM (1..8) */
    int32_t march_inner;   /* SDF evaluations per march lane between the warp's refills (1..16; default 6) */
} pt_wavefront_tuning;
int pt_get_wavefront_tuning(pt_ctx* ctx, pt_wavefront_tuning* out);
int pt_set_wavefront_tuning(pt_ctx* ctx, const pt_wavefront_tuning* tuning);
/* The autotuner: coordinate descent over the knobs above, `rounds` passes,
 * timing wavefront dispatches of `push` (its resolution must be the
 * accumulator's) on the bound scene; a knob moves only for a gain of at least
 * 3 %.  Installs and returns the fastest setting and its seconds per
 * dispatch; the accumulator is left as it was. */
int pt_autotune_wavefront(pt_ctx* ctx, const pt_push* push, int rounds, pt_wavefront_tuning* best,
                          double* best_seconds);

/* Stage timing of the wavefront engine: when on, iterations are launched one
 * kernel at a time with CUDA events around each stage (isect, march, shade,
 * gen, bookkeeping; rays are intersected inside shade and gen, so the isect
 * entry reads 0), and pt_get_stage_times returns the
 * device milliseconds summed per stage since timing was switched on, and the
 * iterations timed.  Off by default (it disables graph replay). */
int pt_set_stage_timing(pt_ctx* ctx, int on);
int pt_get_stage_times(pt_ctx* ctx, double ms[5], uint64_t* iterations);

/* ---------------------------------------------------------------------------
 * Batched rendering.  No counterpart in the reference, which renders one
 * scene per compute dispatch (src/pathtracer.cpp:3586-3608): these calls keep
 * many scenes and accumulators resident on one device and run render passes
 * of all of them through one shared wavefront path pool, so a pass of a small
 * job fills the lanes a large job leaves idle.
 *
 *   scene   a packed pt_ubo plus its SDF plug-ins (as pt_upload_scene +
 *           pt_set_sdf_plugins), copied at call time;
 *   target  an accumulator of W x H pixels: PT_TARGET_FLOAT is the
 *           reference's float4 XYZ buffer (Rendering/Accumulate,
 *           src/shader.comp:1492-1523); PT_TARGET_FP64 sums every sample's
 *           exposed XYZ in double precision (reference images: FP32 paths,
 *           FP64 accumulation; read back as the mean);
 *   pass    one dispatch's worth of samples (a pt_push) of one scene into one
 *           target.  A pass into a float target ends with exactly the value
 *           pt_dispatch would leave for the same push constants, bit for bit.
 *
 * Two engines run the passes, each on its own stream: the staged wavefront
 * kernels (compacted ray queues; best where SDF marching makes lanes
 * diverge) and a persistent path kernel (paths stay in registers, lanes
 * refill from a shared sample counter; best for analytic scenes).  The
 * default route sends passes of scenes with SDFs to the first and the rest
 * to the second; both give results bit-identical to pt_dispatch.
 *
 * Passes are resolved in the order they were added per target; passes of
 * different targets complete independently.  A batch is single-threaded like
 * a context.  pt_batch_step returns the passes that completed (resolved) since
 * the last call; pt_batch_run steps until none is pending.
 * ------------------------------------------------------------------------- */
typedef struct pt_batch pt_batch;

#define PT_TARGET_FLOAT 0
#define PT_TARGET_FP64 1

#define PT_BATCH_ROUTE_AUTO 0       /* SDF scenes staged, analytic scenes persistent */
#define PT_BATCH_ROUTE_STAGED 1     /* every pass through the staged wavefront kernels */
#define PT_BATCH_ROUTE_PERSISTENT 2 /* every pass through the persistent path kernel */

typedef struct pt_batch_info {
    uint64_t samples_done;  /* samples of resolved passes */
    uint64_t samples_added; /* samples of every pass added */
    uint64_t iterations;    /* wavefront iterations launched */
    uint32_t passes_added;
    uint32_t passes_pending;
    uint32_t pool_slots;
    uint32_t pass_slots;    /* passes of one engine that can be in flight at once */
    uint32_t passes_staged; /* passes routed to each engine so far */
    uint32_t passes_persistent;
    uint64_t kernel_launches; /* kernels the batch has launched (graph replays counted per kernel) */
} pt_batch_info;

/* pool_slots >= 1024 paths in flight in each staged engine; max_passes
 * passes of each engine in flight at once. */
int pt_batch_create(pt_batch** out, int device, uint32_t pool_slots, uint32_t max_passes);
int pt_batch_destroy(pt_batch* batch);
const char* pt_batch_last_error(pt_batch* batch);
void* pt_batch_stream(pt_batch* batch);
int pt_batch_set_march_budget(pt_batch* batch, int steps);
/* Idle lanes a warp of the persistent kernel gathers before it starts new
 * samples together (1..32, default 16: starting samples one lane at a time
 * runs the camera and lens code with few lanes active). */
int pt_batch_set_persist_refill(pt_batch* batch, int lanes);
/* Staged engines (1 or 2; default 2) for passes added from now on: with 2, a
 * staged pass of at least 4 * pool_slots samples is split in two halves (in
 * sample order) between two staged engines with a pool each, on two streams,
 * as pt_set_wavefront_engines does for a context; the same bits as one
 * engine.  The second engine's pool is allocated by the first such pass. */
int pt_batch_set_wavefront_engines(pt_batch* batch, int engines);
/* Engine choice for passes added from now on (PT_BATCH_ROUTE_*). */
int pt_batch_set_route(pt_batch* batch, int route);
int pt_batch_add_scene(pt_batch* batch, const pt_ubo* ubo, const pt_sdf_plugin* plugins, int nplugins,
                       int* scene_id);
/* Extensions of an added scene (NULL: the reference's method), used by
 * passes added from now on; PT_ERR_BUSY while passes of the scene are in flight. */
int pt_batch_set_scene_ext(pt_batch* batch, int scene_id, const pt_scene_ext* ext);
/* A scene whose SDFs are given as text, like pt_set_sdfs: the shipped
 * snippets and builtin: specs select plug-ins, any other GLSL is translated
 * here (PT_ERR_UNSUPPORTED with the reason for what the translator cannot
 * express) and compiled with NVRTC, together with every other snippet of the
 * batch, into the staged engine's march kernel before the next step.  Such
 * scenes render on the staged engine (a persistent route is refused). */
int pt_batch_add_scene_sources(pt_batch* batch, const pt_ubo* ubo, const char* const* sources, int n, int* scene_id);
int pt_batch_add_target(pt_batch* batch, int width, int height, int kind, int* target_id);
/* Device pointer of a target: float4 per pixel (FLOAT) or 4 doubles per pixel
 * (FP64: x, y, z sums and the sample count). */
void* pt_batch_target_device_ptr(pt_batch* batch, int target_id);
/* Queues a pass; push->resolution must be the target's.  PT_ERR_BUSY when
 * max_passes passes are in flight. */
int pt_batch_add_pass(pt_batch* batch, int scene_id, int target_id, const pt_push* push, int* pass_id);
/* An FP64 reference pass (no counterpart in the reference): one dispatch's
 * samples (push) of a resident scene traced in double precision by
 * pt_render_fp64's kernel and added to an FP64 target, instead of FP32
 * paths summed in double as a pass does.  Asynchronous on the batch's
 * stream, ordered before every later RMSE reduction of the batch; it is no
 * pass (no pass id, nothing for pt_batch_step to return).  The batch's SDF
 * text compiled at run time is compiled once more for it, in double (the
 * first call after new snippets arrive takes seconds). */
int pt_batch_render_fp64(pt_batch* batch, int scene_id, int target_id, const pt_push* push);
/* pt_set_device_checks for both of the batch's engines; a failed check
 * makes pt_batch_step (and pt_batch_run) return PT_ERR_KERNEL.  PT_ERR_BUSY
 * while passes are in flight. */
int pt_batch_set_device_checks(pt_batch* batch, int on);
int pt_batch_step(pt_batch* batch, int iterations, int* completed, int capacity, int* ncompleted);
int pt_batch_pending(pt_batch* batch);
int pt_batch_run(pt_batch* batch, uint64_t max_iterations);
int pt_batch_stats(pt_batch* batch, pt_batch_info* out);
/* Samples per pixel resolved into a target so far. */
int pt_batch_target_samples(pt_batch* batch, int target_id, uint64_t* samples);
/* W*H float4 (FP64 targets: their mean, rounded to float). */
int pt_batch_read_target(pt_batch* batch, int target_id, float* host, size_t bytes);
/* sqrt(sum |a - r|^2 / sum |r|^2) over the XYZ channels of a float target a
 * against a reference target r of the same size, reduced on the device in
 * double precision. */
int pt_batch_rmse(pt_batch* batch, int target_id, int reference_id, double* rel_rmse);
/* The same for n (target, reference) pairs in one launch and one copy back. */
int pt_batch_rmse_many(pt_batch* batch, const int* target_ids, const int* reference_ids, int n, double* rel_rmse);
/* The same for a caller's device image (W*H float4, e.g. a context's
 * accumulator, complete before the call) against a reference target. */
int pt_batch_rmse_image(pt_batch* batch, const void* d_image, int width, int height, int reference_id,
                        double* rel_rmse);
/* PT_ERR_BUSY while passes of the target / scene are in flight. */
int pt_batch_release_target(pt_batch* batch, int target_id);
int pt_batch_release_scene(pt_batch* batch, int scene_id);

/* Event word layout, identical in the CPU restatement used by the tests. */
#define PT_EV_HIT_MASK 0xFFFu     /* global object index; PT_EV_HIT_SDF, PT_EV_HIT_MISS */
#define PT_EV_HIT_SDF 0xFFEu
#define PT_EV_HIT_MISS 0xFFFu
#define PT_EV_EMITTER (1u << 12)  /* emitter hit, path terminated */
#define PT_EV_LIGHT_SHIFT 13      /* 7 bits: light pick index (randomLight) */
#define PT_EV_SHADOW_SHIFT 20     /* 2 bits: 0 none, 1 RR-culled, 2 occluded, 3 visible */
#define PT_EV_RR_KILL (1u << 22)  /* terminated by Russian roulette */
#define PT_EV_VALID (1u << 23)
#define PT_EV_SPECULAR (1u << 24) /* extension materials: a specular bounce (mirror or dielectric reflection) */
#define PT_EV_REFRACT (1u << 25)  /* extension materials: a dielectric transmission */

#ifdef __cplusplus
}
#endif

#endif /* PT_CUDA_H */
