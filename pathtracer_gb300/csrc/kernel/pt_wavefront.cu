// pt_wavefront.cu — the wavefront renderer: path state in HBM, compacted
// ray queues, a persistent SDF-march kernel with per-lane ray refill.
//
// The plain megakernel keeps one pixel per thread, so lanes wait for the
// slowest neighbour's SDF march and for pixels with more work (measured:
// 5.3 of 32 lanes active per warp instruction).  Here every path sample of a
// dispatch is an independent work item in a pool of P slots; each iteration
// runs three stage kernels over compacted queues:
//   march  persistent: each lane holds one ray and does one SDF evaluation
//          per step (sign probe, march step, normal probes), several steps
//          between refills from the queue, so all lanes execute the same SDF
//          code -> finished rays to this iteration's SHADE queues;
//   shade  shadow-ray results, then primary hits: emitter / miss / BRDF
//          sample / light sample / Russian roulette (the shared pt_path.cuh
//          functions); finished samples write their XYZ and free their slot;
//          the ray a path continues with is intersected at once (analytic
//          primitives, SDF boxes) and goes to the next iteration's MARCH or
//          SHADE queue;
//   gen    start new samples in free slots, intersect their camera rays the
//          same way.
// A one-thread bookkeeping kernel advances the counters.  Queues are filled
// with warp-aggregated atomics (ballot + popc + one atomicAdd per warp).
// After the last sample, `resolve` sums each pixel's samples in sample order
// and applies Rendering/Accumulate — the same float operations, in the same
// order, as the megakernel and the shader, so results are bit-identical.
// The larger pt_mathf functions are called out of line here (smaller stage
// and persistent kernels); the SDF plug-ins use inlined math regardless.
//
// pt_wavefront_checked.cu compiles this file a second time with
// PT_DEBUG_CHECKS (every queue, pool-slot, ring and sample index checked
// before use; pt_check in pt_march.cuh) and its launch functions renamed by
// PTK_WF; the engine picks either set (ptk_wavefront_kernels).
#define PTM_OUTLINE
#include <cuda_runtime.h>

#ifndef PTK_WF
#define PTK_WF(name) name
#endif

#include "pt_march.cuh"
#include "pt_path.cuh"
#include "pt_wavefront.h"

namespace {

// The flags word of s8: bit 30 the shadow-ray flag (kShadowFlag), bits
// 28-29 the extension dielectrics' path bits (PathState::medium), the bounce
// count below.
constexpr uint32_t kMediumShift = 28;
constexpr uint32_t kBounceMask = (1u << kMediumShift) - 1u;
PT_DI uint32_t bounce_word(const PathState& ps) {
    return ((uint32_t)ps.medium << kMediumShift) | ((uint32_t)ps.bounce & kBounceMask);
}

// A shadow-ray result's state: the bounce's next ray (s0, s1), the NEE
// term and the next throughput made with the shadow ray (s3, s5: see
// shade_shadow_made), the radiance, wavelengths and RNG/pass words and,
// traced, the event word.  The light sample's geometry and the BRDF those
// two came from are not stored, so they are neither read here.
template <bool TRACE>
PT_DI void load_for_shadow(const PoolView& v, uint32_t slot, PathState& ps, float4& contrib, uint32_t& flags,
                           uint32_t& sample, uint32_t& job) {
    const float4 a = v.s0[slot], b = v.s1[slot];
    ps.org = f3(a.x, a.y, a.z);
    ps.mis = a.w;
    ps.dir = f3(b.x, b.y, b.z);
    ps.brdfPdf = b.w;
    ps.shDir = f3(0.0f, 0.0f, 0.0f);
    ps.cosL = 0.0f;
    ps.nrm = f3(0.0f, 0.0f, 0.0f);
    ps.lightPdf = 0.0f;
    ps.brdf = f4s(0.0f);
    contrib = v.s3[slot];
    ps.rr = v.s5[slot];
    ps.radiance = v.s6[slot];
    ps.l = v.s7[slot];
    const uint4 m = v.s8[slot];
    ps.seed = m.x;
    flags = m.y;
    ps.bounce = (int)(m.y & kBounceMask);
    ps.medium = (int)((m.y >> kMediumShift) & 3u);
    sample = m.z;
    ps.shObj = word_shobj(m.w);
    job = word_job(m.w);
    if (TRACE) {
        const float4 e = v.s9[slot];
        ps.shLightID = e.x;
        ps.ev = __float_as_uint(e.y);
    } else {
        ps.shLightID = -1.0f;
        ps.ev = 0u;
    }
}

// A new sample's state.  Its first step is a primary ray (march, then
// shade_primary), which reads neither the shadow-ray fields (s2, s3), the
// BRDF (s4) nor the light pick (s9.x) and writes what a shadow ray reads
// before it reads it; at bounce 0 the throughput, the radiance and the event word
// are start_sample's constants (1, 0, 0), which load_for_primary sets
// instead of reading s5, s6 and s9.  So only s0, s1, s7 and s8 are stored.
PT_DI void store_new_sample(const PoolView& v, uint32_t slot, const PathState& ps, uint32_t sample, uint32_t job) {
    v.s0[slot] = make_float4(ps.org.x, ps.org.y, ps.org.z, ps.mis);
    v.s1[slot] = make_float4(ps.dir.x, ps.dir.y, ps.dir.z, ps.brdfPdf);
    v.s7[slot] = ps.l;
    v.s8[slot] = make_uint4(ps.seed, bounce_word(ps), sample, job_word(job, ps.shObj));
}

// The ring entry of the pass that holds global sample s: the last pass in
// [lo, hi) with first <= s (passes are appended in increasing order of first).
PT_DI uint32_t find_job(const WfJob* __restrict__ jobs, uint32_t cap, uint32_t lo, uint32_t hi, uint64_t s) {
    // invariant: jobs[lo % cap].first <= s < jobs[hi % cap].first (or hi is the end)
    while (hi - lo > 1) {
        const uint32_t mid = lo + ((hi - lo) >> 1);
        if (jobs[mid % cap].first <= s) {
            lo = mid;
        } else {
            hi = mid;
        }
    }
    return lo % cap;
}

// Sample id s of a dispatch: k = s / (W*H), pixel = s % (W*H).  The colour
// buffer is [k][pixel], so `resolve` reads it coalesced; traces use the
// megakernel's path index pixel * spf + k.
PT_DI size_t trace_index(const pt_push& pc, uint32_t s) {
    const uint32_t npix = (uint32_t)pc.resolution[0] * (uint32_t)pc.resolution[1];
    return (size_t)(s % npix) * (size_t)pc.samplesPerFrame + (size_t)(s / npix);
}

// Samples of every pass added so far: the end of the last pass.
PT_DI uint64_t jobs_total(const WfArgs& A, uint32_t hi) {
    if (hi == 0) return 0;
    const WfJob& L = A.jobs[(hi - 1) % A.job_cap];
    return L.first + (uint64_t)L.count;
}

// Intersection for a ray a stage has just produced (the reference's
// Intersection up to SphereTracing, SC:862-923 and SC:779-790): analytic
// primitives, then the SDF bounding boxes.  Writes the hit record and, for a
// ray that needs sphere tracing, the march start state (the march kernel
// picks it up like a ray it suspended).  Returns true for such a ray.
PT_DI bool route_ray(const WfArgs& A, const PoolView& v, const KScene& S, uint32_t slot, float3 org, float3 dir) {
    Hit h;
    h.hitdist = PT_MAXDIST;
    h.normal = f3(0.0f, 0.0f, 0.0f);
    h.materialID = 0.0f;
    h.lightID = -1.0f;
    int objectID = -1;
    intersect_analytic(S, org, dir, h, objectID);
    bool march = false;
    if (S.meta.n[5] > 0) {
        const float3 invdir = f3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
        float2 tmm = make_float2(PT_MAXDIST, PT_MAXDIST);
        uint32_t set1 = 0;
        march = search_sdf(S, org, invdir, tmm, set1);
        if (march) {
            v.m0[slot] = make_float4(fmaxf(tmm.x, 1e-3f), 0.0f, kOmegaMax, 0.0f);
            v.m1[slot] = make_float4(tmm.x, tmm.y, __uint_as_float(0u), __uint_as_float(set1));  // not suspended
        }
    }
    v.h0[slot] = make_float4(h.hitdist, h.materialID, h.lightID, __int_as_float(objectID));
    v.h1[slot] = make_float4(h.normal.x, h.normal.y, h.normal.z, 0.0f);
    return march;
}

// Appends a routed ray to the next iteration's queues: march, or shading of
// a primary hit or of a shadow-ray result.  Called by all 32 lanes.
PT_DI void push_routed(const WfArgs& A, WfCounters& C, uint32_t nxt, uint32_t slot, bool valid, bool march,
                       bool shadow_ray) {
    q_push(A, A.q_march[nxt], &C.n_march[nxt], slot, valid && march);
    q_push(A, A.q_shade[nxt], &C.n_shade[nxt], slot, valid && !march && !shadow_ray);
    q_push(A, A.q_shadow[nxt], &C.n_shadow[nxt], slot, valid && !march && shadow_ray);
}

__global__ void PT_GEN_BOUNDS wf_gen(const __grid_constant__ WfArgs A) {
    WfCounters& C = *A.counters;
    const uint32_t job_lo = C.job_lo, job_hi = C.job_hi;
    const uint64_t remaining = jobs_total(A, job_hi) - C.next_sample;
    const uint32_t n = (uint32_t)min((uint64_t)C.n_free, remaining);
    const uint32_t nfree = C.n_free;
    const uint64_t first = C.next_sample;
    const uint32_t nxt = C.cur ^ 1u;
    const PoolView v = view(A);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t i = base + threadIdx.x;
        bool valid = i < n;
        uint32_t slot = 0;
        bool march = false;
        if (valid) valid = pt_check(A, nfree - n + i, A.pool_size, PT_CHECK_FREE_INDEX);
        if (valid) {
            slot = A.q_free[nfree - n + i];
            valid = pt_check(A, slot, A.pool_size, PT_CHECK_QUEUE_SLOT);
        }
        if (valid) {
            const uint64_t s = first + i;
            const uint32_t job = find_job(A.jobs, A.job_cap, job_lo, job_hi, s);
            const WfJob& J = A.jobs[job];
            const uint32_t local = J.local_base + (uint32_t)(s - J.first);
            const pt_push& pc = J.pc;
            const int W = pc.resolution[0], H = pc.resolution[1];
            const uint32_t npix = (uint32_t)W * (uint32_t)H;
            const uint32_t k = local / npix, pix = local % npix;
            const int x = (int)(pix % (uint32_t)W), y = (int)(pix / (uint32_t)W);
            const uint32_t xx = (uint32_t)x, yy = (uint32_t)H - (uint32_t)y;
            const float uvx = (2.0f * (float)xx - (float)W) / (float)H;
            const float uvy = (2.0f * (float)yy - (float)H) / (float)H;
            const CamInfo cam = J.cam;
            PathState ps;
            start_sample(ps, *J.scene, pc, cam, xx, yy, uvx, uvy, (int)k);
            ps.brdfPdf = 0.0f;
            ps.shLightID = -1.0f;
            ps.shObj = 0;
            ps.ev = 0;
            store_new_sample(v, slot, ps, local, job);
            march = route_ray(A, v, *J.scene, slot, ps.org, ps.dir);
        }
        push_routed(A, C, nxt, slot, valid, march, false);
    }
}

__global__ void wf_job_add(const __grid_constant__ WfArgs A, const WfJob job, uint32_t index, uint32_t lo) {
    WfJob& J = A.jobs[index % A.job_cap];
    J = job;
    J.finished = 0;
    J.cam = make_camera(job.pc);
    WfCounters& C = *A.counters;
    C.job_hi = index + 1;
    C.job_lo = lo;
}

// Adds 1 to jobs[job].finished for every lane with pred, one atomic per
// distinct job in the warp.  Called by all 32 lanes.
PT_DI void count_finished(WfJob* __restrict__ jobs, uint32_t job, bool pred) {
    const unsigned active = __ballot_sync(0xffffffffu, pred);
    if (!active) return;
    const unsigned same = __match_any_sync(0xffffffffu, pred ? job : 0xffffffffu);
    if (pred && (__ffs(same & active) - 1) == (int)(threadIdx.x & 31))
        atomicAdd(&jobs[job].finished, (uint32_t)__popc(same & active));
}

// A primary hit reads neither the shadow-ray fields (s2, s3) nor the BRDF
// (s4): it writes them.
template <bool TRACE>
PT_DI void load_for_primary(const PoolView& v, uint32_t slot, PathState& ps, uint32_t& flags, uint32_t& sample,
                            uint32_t& job) {
    const float4 a = v.s0[slot], b = v.s1[slot];
    ps.org = f3(a.x, a.y, a.z);
    ps.mis = a.w;
    ps.dir = f3(b.x, b.y, b.z);
    ps.brdfPdf = b.w;
    ps.shDir = f3(0.0f, 0.0f, 0.0f);
    ps.cosL = 0.0f;
    ps.nrm = f3(0.0f, 0.0f, 0.0f);
    ps.lightPdf = 0.0f;
    ps.brdf = f4s(0.0f);
    ps.l = v.s7[slot];
    const uint4 m = v.s8[slot];
    ps.seed = m.x;
    flags = m.y;
    ps.bounce = (int)(m.y & kBounceMask);
    ps.medium = (int)((m.y >> kMediumShift) & 3u);
    sample = m.z;
    ps.shObj = word_shobj(m.w);
    job = word_job(m.w);
    // A first hit (bounce 0) has start_sample's throughput 1, radiance 0 and
    // no events yet (store_new_sample stores none of them).  s9 holds the
    // light pick and the event word, which only a traced dispatch keeps.
    if (ps.bounce == 0) {
        ps.rr = f4s(1.0f);
        ps.radiance = f4s(0.0f);
        ps.ev = 0u;
    } else {
        ps.rr = v.s5[slot];
        ps.radiance = v.s6[slot];
        ps.ev = TRACE ? __float_as_uint(v.s9[slot].y) : 0u;
    }
    ps.shLightID = -1.0f;
}

// After a shadow-ray result only the throughput, the radiance, the RNG and
// bounce word and (traced) the event word change.  The wavelengths (s7)
// never change but are stored with s8 so the pair's sector is written
// whole (a partial sector write makes the L2 read the rest from DRAM).
PT_DI void store_after_shadow(const PoolView& v, uint32_t slot, const PathState& ps, uint32_t sample, uint32_t job,
                              bool trace) {
    v.s5[slot] = ps.rr;
    v.s6[slot] = ps.radiance;
    v.s7[slot] = ps.l;
    v.s8[slot] = make_uint4(ps.seed, bounce_word(ps), sample, job_word(job, ps.shObj));
    if (trace) v.s9[slot] = make_float4(ps.shLightID, __uint_as_float(ps.ev), 0.0f, 0.0f);
}

// The end of a shaded step: trace records, the sample's colour when the
// path ended, the queues.
template <bool TRACE>
PT_DI void finish_shade(const WfArgs& A, const WfJob& J, const PathState& ps, StepResult r, uint32_t sample,
                        bool& freed) {
    const pt_push& pc = J.pc;
    // trace and colour indices
    const bool in_pass = pt_check(A, sample - J.local_base, J.count, PT_CHECK_SAMPLE);
    if (TRACE && r != STEP_SHADOW && A.trace.events && in_pass) {
        const size_t p = trace_index(pc, sample);
        const int b = ps.bounce - 1;
        if (b < A.trace.cap) A.trace.events[p * (size_t)A.trace.cap + b] = ps.ev;
    }
    if (r == STEP_TERMINATED && !in_pass) {
        freed = true;
    } else if (r == STEP_TERMINATED) {
        const float3 col = sample_color(ps, *J.scene, J.cie);
        J.colors[sample] = make_float4(col.x, col.y, col.z, 0.0f);
        if (TRACE) {
            const size_t p = trace_index(pc, sample);
            if (A.trace.nevents) A.trace.nevents[p] = (uint32_t)ps.bounce;
            if (A.trace.colors) {
                A.trace.colors[3 * p] = col.x;
                A.trace.colors[3 * p + 1] = col.y;
                A.trace.colors[3 * p + 2] = col.z;
            }
        }
        freed = true;
    }
}

// Shading in two passes over two queues, so each warp runs one kind of step
// and moves only the state that kind reads and writes: shadow-ray results
// (the light sample's contribution, then the bounce's end), then primary
// hits (emission or BRDF and light sampling).
template <bool TRACE>
__global__ void PT_SHADE_BOUNDS wf_shade(const __grid_constant__ WfArgs A) {
    WfCounters& C = *A.counters;
    const uint32_t cur = C.cur, nxt = cur ^ 1u;
    const PoolView v = view(A);
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t ns = C.n_shadow[cur];
    for (uint32_t base = blockIdx.x * blockDim.x; base < ns; base += stride) {
        const uint32_t i = base + threadIdx.x;
        bool valid = i < ns;
        uint32_t slot = 0, job = 0;
        bool again = false, freed = false, march = false;
        if (valid) {
            slot = A.q_shadow[cur][i];
            valid = pt_check(A, slot, A.pool_size, PT_CHECK_QUEUE_SLOT) &&
                    pt_check(A, slot_job(v, slot), A.job_cap, PT_CHECK_JOB);
        }
        if (valid) {
            PathState ps;
            float4 contrib;
            uint32_t flags, sample;
            load_for_shadow<TRACE>(v, slot, ps, contrib, flags, sample, job);
            const WfJob& J = A.jobs[job];
            const int objectID = __float_as_int(v.h0[slot].w);
            const float4 rr_next = ps.rr;
            const StepResult r = shade_shadow_made<TRACE>(ps, objectID, contrib, rr_next, J.pc.pathLength);
            finish_shade<TRACE>(A, J, ps, r, sample, freed);
            if (!freed) {
                store_after_shadow(v, slot, ps, sample, job, TRACE);
                again = true;
                // the bounce's next primary ray, set up with the primary hit
                march = route_ray(A, v, *J.scene, slot, ps.org, ps.dir);
            }
        }
        push_routed(A, C, nxt, slot, again, march, false);
        q_push(A, A.q_free, &C.n_free, slot, freed);
        count_finished(A.jobs, job, freed);
    }
    const uint32_t np = C.n_shade[cur];
    for (uint32_t base = blockIdx.x * blockDim.x; base < np; base += stride) {
        const uint32_t i = base + threadIdx.x;
        bool valid = i < np;
        uint32_t slot = 0, job = 0;
        bool again = false, freed = false, march = false, shadow_next = false;
        if (valid) {
            slot = A.q_shade[cur][i];
            valid = pt_check(A, slot, A.pool_size, PT_CHECK_QUEUE_SLOT) &&
                    pt_check(A, slot_job(v, slot), A.job_cap, PT_CHECK_JOB);
        }
        if (valid) {
            PathState ps;
            uint32_t flags, sample;
            load_for_primary<TRACE>(v, slot, ps, flags, sample, job);
            const WfJob& J = A.jobs[job];
            const float4 h0 = v.h0[slot], h1 = v.h1[slot];
            Hit h;
            h.hitdist = h0.x;
            h.materialID = h0.y;
            h.lightID = h0.z;
            h.normal = f3(h1.x, h1.y, h1.z);
            const int objectID = __float_as_int(h0.w);
            const StepResult r = shade_primary<TRACE>(ps, *J.scene, h, objectID, J.pc.pathLength);
            finish_shade<TRACE>(A, J, ps, r, sample, freed);
            if (!freed) {
                // the path state.  For a light sample's shadow ray: its
                // direction (s2, read by the march) and, made now with the
                // shadow step's own operations (shade_shadow_made), the NEE
                // term (s3) and the bounce's next throughput (s5), so the
                // shadow step reads neither the light sample's geometry nor
                // the BRDF (s4 is kept only when traced, beside s9).  A next
                // bounce's primary ray reads none of s2-s4.
                v.s0[slot] = make_float4(ps.org.x, ps.org.y, ps.org.z, ps.mis);
                v.s1[slot] = make_float4(ps.dir.x, ps.dir.y, ps.dir.z, ps.brdfPdf);
                if (r == STEP_SHADOW) {
                    v.s2[slot] = make_float4(ps.shDir.x, ps.shDir.y, ps.shDir.z, ps.cosL);
                    v.s3[slot] = shadow_contribution(ps, *J.scene);
                    if (TRACE) v.s4[slot] = ps.brdf;
                }
                v.s5[slot] = (r == STEP_SHADOW) ? bounce_throughput(ps) : ps.rr;
                v.s6[slot] = ps.radiance;
                v.s7[slot] = ps.l;  // unchanged: written with s8 so their sector is written whole
                v.s8[slot] = make_uint4(ps.seed, ((r == STEP_SHADOW) ? kShadowFlag : 0u) | bounce_word(ps), sample,
                                        job_word(job, ps.shObj));
                // traced: the light picked and the event word
                if (TRACE) v.s9[slot] = make_float4(ps.shLightID, __uint_as_float(ps.ev), 0.0f, 0.0f);
                again = true;
                // the light sample's shadow ray, or the next bounce
                shadow_next = (r == STEP_SHADOW);
                march = route_ray(A, v, *J.scene, slot, ps.org, shadow_next ? ps.shDir : ps.dir);
            }
        }
        push_routed(A, C, nxt, slot, again, march, shadow_next);
        q_push(A, A.q_free, &C.n_free, slot, freed);
        count_finished(A.jobs, job, freed);
    }
}

// Persistent mode: the megakernel's per-thread path loop (one intersect_all
// call site per iteration for primary and shadow rays alike) over the samples
// of every pass in the ring.  A lane whose path ends takes the next sample
// at once, from a chunk its warp claimed with one atomic, so lanes stay busy
// across pixels, samples and passes; no path state leaves registers.  Each
// sample's colour goes to its pass's colour buffer, which `resolve` sums in
// sample order, so results equal the megakernel's bit for bit.  Suited to
// scenes without SDFs, where lanes of a warp do similar work per ray; SDF
// marching diverges per lane and belongs to the staged kernels above.
constexpr uint32_t kPersistChunk = 256;

__global__ void wf_persist_setup(const __grid_constant__ WfArgs A, uint64_t budget) {
    WfCounters& C = *A.counters;
    const uint64_t total = jobs_total(A, C.job_hi);
    const uint64_t begin = C.pk_end;  // warps of the last launch may have claimed past it
    const uint64_t end = (total - begin > budget) ? begin + budget : total;
    C.next_sample = begin;
    C.pk_end = end;
    C.total = total;
    C.iterations += 1;
}

// The persistent path loop.  ONE: every sample of the launch belongs to one
// pass, whose scene S1 is the launch's parameter (the constant bank, as
// for the megakernel); otherwise each lane reads its pass's scene through
// the pass's pointer.
template <int FEAT, bool ONE>
PT_DI void persist_paths(const WfArgs& A, const KScene* S1) {
    WfCounters& C = *A.counters;
    const uint64_t end = C.pk_end;
    const uint32_t job_lo = C.job_lo, job_hi = C.job_hi;
    const int lane = (int)(threadIdx.x & 31);
    const unsigned lt = (1u << lane) - 1u;
    uint64_t cbase = 0;   // warp-uniform: unassigned samples of the warp's chunk
    uint32_t cleft = 0;
    uint32_t cjob = 0;      // warp-uniform: pass of the chunk's first sample,
    uint64_t cjob_end = 0;  // and the end of its sample range
    bool exhausted = false;  // warp-uniform: no sample left below `end`
    bool active = false, shadow = false;
    uint32_t job = 0, local = 0;
    PathState ps;
    for (;;) {
        // Refill idle lanes from the warp's chunk, claiming chunks as needed,
        // once persist_refill lanes are idle (or none is busy): new samples
        // start together instead of one lane at a time.
        unsigned need = __ballot_sync(0xffffffffu, !active);
        if (__popc(need) < A.persist_refill && need != 0xffffffffu) need = 0u;
        while (need && !exhausted) {
            if (cleft == 0) {
                unsigned long long b = 0;
                if (lane == 0) b = atomicAdd(reinterpret_cast<unsigned long long*>(&C.next_sample), kPersistChunk);
                b = __shfl_sync(0xffffffffu, b, 0);
                if (b >= end) {
                    exhausted = true;
                    break;
                }
                cbase = b;
                cleft = (end - b < kPersistChunk) ? (uint32_t)(end - b) : kPersistChunk;
                // The pass of the chunk's first sample, looked up once for the warp.
                uint32_t cj = 0;
                if (lane == 0) cj = find_job(A.jobs, A.job_cap, job_lo, job_hi, b);
                cjob = __shfl_sync(0xffffffffu, cj, 0);
                const WfJob& CJ = A.jobs[cjob];
                cjob_end = CJ.first + (uint64_t)CJ.count;
            }
            const uint32_t n = min((uint32_t)__popc(need), cleft);
            const uint32_t rank = (uint32_t)__popc(need & lt);
            const bool mine = ((need >> lane) & 1u) && rank < n;
            if (mine) {
                const uint64_t s = cbase + rank;
                job = (s < cjob_end) ? cjob : find_job(A.jobs, A.job_cap, job_lo, job_hi, s);
                const WfJob& J = A.jobs[job];
                local = J.local_base + (uint32_t)(s - J.first);
                const pt_push& pc = J.pc;
                const int W = pc.resolution[0], H = pc.resolution[1];
                const uint32_t npix = (uint32_t)W * (uint32_t)H;
                const uint32_t k = local / npix, pix = local % npix;
                const uint32_t xx = pix % (uint32_t)W, yy = (uint32_t)H - pix / (uint32_t)W;
                const float uvx = (2.0f * (float)xx - (float)W) / (float)H;
                const float uvy = (2.0f * (float)yy - (float)H) / (float)H;
                const CamInfo cam = J.cam;
                start_sample(ps, ONE ? *S1 : *J.scene, pc, cam, xx, yy, uvx, uvy, (int)k);
                shadow = false;
                active = true;
            }
            cbase += n;
            cleft -= n;
            need = __ballot_sync(0xffffffffu, !active);
        }
        if (exhausted && __ballot_sync(0xffffffffu, active) == 0) break;
        bool finished = false;
        if (active) {
            const WfJob& J = A.jobs[job];
            const KScene& S = ONE ? *S1 : *J.scene;
            const int depth = J.pc.pathLength;
            Hit h;
            h.hitdist = PT_MAXDIST;
            h.normal = f3(0.0f, 0.0f, 0.0f);
            h.materialID = 0.0f;
            h.lightID = -1.0f;
            int objectID = -1;
            intersect_all<FEAT>(S, ps.org, shadow ? ps.shDir : ps.dir, h, objectID);
            const StepResult r = shadow ? shade_shadow<false>(ps, S, objectID, depth)
                                        : shade_primary<false>(ps, S, h, objectID, depth);
            shadow = (r == STEP_SHADOW);
            if (r == STEP_TERMINATED) {
                const float3 col = sample_color(ps, S, J.cie);
                if (pt_check(A, local - J.local_base, J.count, PT_CHECK_SAMPLE))
                    J.colors[local] = make_float4(col.x, col.y, col.z, 0.0f);
                finished = true;
                active = false;
            }
        }
        count_finished(A.jobs, job, finished);
    }
}

template <int FEAT>
__global__ void __launch_bounds__(kPersistThreads) wf_persist(const __grid_constant__ WfArgs A) {
    persist_paths<FEAT, false>(A, nullptr);
}

template <int FEAT>
__global__ void __launch_bounds__(kPersistThreads)
    wf_persist_one(const __grid_constant__ WfArgs A, const __grid_constant__ KScene S1) {
    persist_paths<FEAT, true>(A, &S1);
}

__global__ void wf_book(const __grid_constant__ WfArgs A) {
    WfCounters& C = *A.counters;
    const uint32_t pool = A.pool_size;
    const uint64_t total = jobs_total(A, C.job_hi);
    const uint32_t n = (uint32_t)min((uint64_t)C.n_free, total - C.next_sample);
    C.total = total;
    C.next_sample += n;
    C.n_free -= n;
    C.n_march[C.cur] = 0;
    C.n_shade[C.cur] = 0;
    C.n_shadow[C.cur] = 0;
    C.cur ^= 1u;
    C.march_cursor = 0;
    C.iterations += 1;
    C.live = pool - C.n_free;
    // the next iteration's queues and the free list fit the pool
    const uint32_t c = C.cur;
    (void)(pt_check(A, C.n_march[c], pool + 1u, PT_CHECK_QUEUE_COUNT) &&
           pt_check(A, C.n_shade[c], pool + 1u, PT_CHECK_QUEUE_COUNT) &&
           pt_check(A, C.n_shadow[c], pool + 1u, PT_CHECK_QUEUE_COUNT) &&
           pt_check(A, C.n_free, pool + 1u, PT_CHECK_QUEUE_COUNT));
}

__global__ void wf_init(WfCounters* __restrict__ Cp, uint32_t* __restrict__ q_free, uint32_t pool) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < pool) q_free[i] = i;
    if (i == 0) {
        WfCounters& C = *Cp;
        C.n_march[0] = C.n_march[1] = 0;
        C.n_shade[0] = C.n_shade[1] = 0;
        C.n_shadow[0] = C.n_shadow[1] = 0;
        C.cur = 0;
        C.march_cursor = 0;
        C.n_free = pool;
        C.next_sample = 0;
        C.total = 0;
        C.iterations = 0;
        C.live = 0;
        C.job_lo = C.job_hi = 0;
        C.pk_end = 0;
        C.check_site = 0;
        C.check_index = 0;
    }
}

// Rendering + Accumulate over one pass's ordered sample colours, one thread per pixel.
__global__ void __launch_bounds__(kStageThreads) wf_resolve(const pt_push pc, float4* __restrict__ accum,
                                                           const float4* __restrict__ colors) {
    const uint32_t npix = (uint32_t)pc.resolution[0] * (uint32_t)pc.resolution[1];
    const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
    if (pix >= npix) return;
    float3 sum = f3(0.0f, 0.0f, 0.0f);
    for (int k = 0; k < pc.samplesPerFrame; k++) {
        const float4 c = colors[(size_t)k * npix + pix];
        sum = sum + f3(c.x, c.y, c.z);
    }
    accum[pix] = accumulate(pc, sum, accum[pix]);
}

}  // namespace

cudaError_t PTK_WF(ptk_wavefront_launch_init)(const WfArgs* a, cudaStream_t stream) {
    wf_init<<<(a->pool_size + 255) / 256, 256, 0, stream>>>(a->counters, a->q_free, a->pool_size);
    return cudaGetLastError();
}

cudaError_t PTK_WF(ptk_wavefront_launch_job_add)(const WfArgs* a, const WfJob* job, uint32_t index, uint32_t lo,
                                         cudaStream_t stream) {
    wf_job_add<<<1, 1, 0, stream>>>(*a, *job, index, lo);
    return cudaGetLastError();
}

// Blocks of a stage kernel resident on the device at once (SMs x the
// kernel's occupancy), cached per kernel: a grid beyond it would leave its
// last blocks for a second wave.
static int resident_blocks(const void* kernel, int* cache) {
    if (*cache) return *cache;
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kStageThreads, 0) != cudaSuccess ||
        per_sm <= 0)
        return 1 << 30;  // unknown: no cap
    *cache = sms * per_sm;
    return *cache;
}

const void* PTK_WF(ptk_wavefront_march_warp_normals)() {
    return reinterpret_cast<const void*>(wf_march_warp_normals);
}

cudaError_t PTK_WF(ptk_wavefront_launch_iteration)(const WfArgs* a, bool trace, int grid, cudaStream_t stream,
                                           cudaEvent_t* stage_events, const void* march_kernel) {
    // stage_events (optional): 6 events recorded before isect, march, shade,
    // gen, bookkeeping and after it, for per-stage device times.
    // (Intersection is done by shade and gen for the rays they produce: the
    // isect interval stays empty.)
    if (stage_events) cudaEventRecord(stage_events[0], stream);
    if (stage_events) cudaEventRecord(stage_events[1], stream);
    if (march_kernel) {
        void* argv[] = {const_cast<WfArgs*>(a)};
        const cudaError_t e = cudaLaunchKernel(march_kernel, dim3(grid), dim3(kStageThreads), argv, 0, stream);
        if (e != cudaSuccess) return e;
    } else {
        wf_march<<<grid, kStageThreads, 0, stream>>>(*a);
    }
    if (stage_events) cudaEventRecord(stage_events[2], stream);
    static int shade_cap[2] = {0, 0}, gen_cap = 0;
    if (trace) {
        const int g = min(grid, resident_blocks(reinterpret_cast<const void*>(wf_shade<true>), &shade_cap[1]));
        wf_shade<true><<<g, kStageThreads, 0, stream>>>(*a);
    } else {
        const int g = min(grid, resident_blocks(reinterpret_cast<const void*>(wf_shade<false>), &shade_cap[0]));
        wf_shade<false><<<g, kStageThreads, 0, stream>>>(*a);
    }
    if (stage_events) cudaEventRecord(stage_events[3], stream);
    wf_gen<<<min(grid, resident_blocks(reinterpret_cast<const void*>(wf_gen), &gen_cap)), kStageThreads, 0,
             stream>>>(*a);
    if (stage_events) cudaEventRecord(stage_events[4], stream);
    wf_book<<<1, 1, 0, stream>>>(*a);
    if (stage_events) cudaEventRecord(stage_events[5], stream);
    return cudaGetLastError();
}

namespace {

// Blocks of a persistent kernel that fit on one SM at once, cached.
template <int FEAT, bool ONE>
int persist_blocks() {
    static int cache = 0;
    if (cache) return cache;
    int n = 0;
    const void* k = ONE ? reinterpret_cast<const void*>(wf_persist_one<FEAT>)
                        : reinterpret_cast<const void*>(wf_persist<FEAT>);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kPersistThreads, 0) != cudaSuccess || n < 1) n = 1;
    cache = n;
    return n;
}

template <int FEAT>
void launch_persist(const WfArgs* a, int sms, const KScene* one_scene, cudaStream_t stream) {
    if (one_scene) {
        wf_persist_one<FEAT><<<sms * persist_blocks<FEAT, true>(), kPersistThreads, 0, stream>>>(*a, *one_scene);
    } else {
        wf_persist<FEAT><<<sms * persist_blocks<FEAT, false>(), kPersistThreads, 0, stream>>>(*a);
    }
}

}  // namespace

cudaError_t PTK_WF(ptk_persist_launch)(const WfArgs* a, int variant, int sms, uint64_t budget,
                                       const KScene* one_scene, cudaStream_t stream) {
    wf_persist_setup<<<1, 1, 0, stream>>>(*a, budget);
    switch (variant) {
        case 0: launch_persist<0>(a, sms, one_scene, stream); break;
        case PT_FEAT_BOX: launch_persist<PT_FEAT_BOX>(a, sms, one_scene, stream); break;
        case PT_FEAT_ANALYTIC: launch_persist<PT_FEAT_ANALYTIC>(a, sms, one_scene, stream); break;
        default: launch_persist<PT_FEAT_ALL>(a, sms, one_scene, stream); break;
    }
    return cudaGetLastError();
}

int PTK_WF(ptk_persist_blocks_per_sm)(int variant) {
    switch (variant & 15) {
        case 0: return persist_blocks<0, false>();
        case PT_FEAT_BOX: return persist_blocks<PT_FEAT_BOX, false>();
        case PT_FEAT_ANALYTIC: return persist_blocks<PT_FEAT_ANALYTIC, false>();
        default: return persist_blocks<PT_FEAT_ALL, false>();
    }
}

cudaError_t PTK_WF(ptk_wavefront_launch_resolve)(const WfArgs* a, uint32_t job, const pt_push* pc, float4* accum,
                                         const float4* colors, cudaStream_t stream) {
    (void)a;
    (void)job;
    const uint32_t npix = (uint32_t)pc->resolution[0] * (uint32_t)pc->resolution[1];
    wf_resolve<<<(npix + kStageThreads - 1) / kStageThreads, kStageThreads, 0, stream>>>(*pc, accum, colors);
    return cudaGetLastError();
}

extern const WfKernelSet PTK_WF(ptk_wavefront_kernel_set);
const WfKernelSet PTK_WF(ptk_wavefront_kernel_set) = {
    PTK_WF(ptk_wavefront_launch_init),        PTK_WF(ptk_wavefront_launch_job_add),
    PTK_WF(ptk_wavefront_launch_iteration),   PTK_WF(ptk_wavefront_march_warp_normals),
    PTK_WF(ptk_persist_launch),               PTK_WF(ptk_persist_blocks_per_sm),
    PTK_WF(ptk_wavefront_launch_resolve),
};
