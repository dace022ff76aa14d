// pt_march.cuh — the wavefront engine's SDF march kernels (wf_march, and
// wf_march_warp_normals for dispatches with a mandelbulb) and the helpers
// every stage kernel shares.  Included by pt_wavefront.cu and, for
// scenes whose SDF text is compiled at run time, by the NVRTC program of
// pt_jit.cu (with PT_JIT_USER_SDF, in namespace ptjit), so both builds run
// the same source.
#pragma once

#include "pt_path.cuh"
#include "pt_wavefront.h"

#if defined(PT_JIT_USER_SDF)
namespace ptjit {
#else
namespace {
#endif

constexpr uint32_t kShadowFlag = 1u << 30;
constexpr int kStageThreads = 256;
// Launch bounds of the stage kernels: resident blocks of kStageThreads per SM
// asked of the compiler (registers capped at 65536 / (256 x blocks)); the
// host caps each kernel's grid at what is resident.  Measured on GB300: the
// march kernel at 4 blocks (64 registers) and shade and gen, which also
// intersect the rays they produce, at 3 (85 registers, no spills) are 1-12 %
// faster end to end than the neighbouring choices.  PT_WF_<STAGE>_BLOCKS
// overrides a count; 0 leaves only the block size.
#ifndef PT_WF_SHADE_BLOCKS
#define PT_WF_SHADE_BLOCKS 3
#endif
#ifndef PT_WF_MARCH_BLOCKS
#define PT_WF_MARCH_BLOCKS 4
#endif
#ifndef PT_WF_GEN_BLOCKS
#define PT_WF_GEN_BLOCKS 3
#endif
#if PT_WF_SHADE_BLOCKS > 0
#define PT_SHADE_BOUNDS __launch_bounds__(kStageThreads, PT_WF_SHADE_BLOCKS)
#else
#define PT_SHADE_BOUNDS __launch_bounds__(kStageThreads)
#endif
#if PT_WF_MARCH_BLOCKS > 0
#define PT_MARCH_BOUNDS __launch_bounds__(kStageThreads, PT_WF_MARCH_BLOCKS)
#else
#define PT_MARCH_BOUNDS __launch_bounds__(kStageThreads)
#endif
#if PT_WF_GEN_BLOCKS > 0
#define PT_GEN_BOUNDS __launch_bounds__(kStageThreads, PT_WF_GEN_BLOCKS)
#else
#define PT_GEN_BOUNDS __launch_bounds__(kStageThreads)
#endif
// wf_march: after a large queue is drained, a warp with fewer rays than
// WfArgs::drain_lanes suspends those that have marched kDrainMinSteps steps
// in this launch, for the next iteration.
constexpr int kDrainMinSteps = 8;

// SphereTracing's over-relaxation start (SC:781).
constexpr float kOmegaMax = 1.70f;

// Index checks of the checked build (PT_DEBUG_CHECKS, the kernels of
// pt_wavefront_checked.cu and checked run-time compiled march kernels):
// true when i < n; otherwise the first failure since the last reset is
// recorded in the counters (site, index) for the host, and the caller skips
// the access.  The default build checks nothing: the function is constant
// true and its arguments are dead code.
#if defined(PT_DEBUG_CHECKS)
PT_DI bool pt_check(const WfArgs& A, uint32_t i, uint32_t n, uint32_t site) {
    if (i < n) return true;
    if (atomicCAS(&A.counters->check_site, 0u, site) == 0u) A.counters->check_index = i;
    return false;
}
#else
PT_DI constexpr bool pt_check(const WfArgs&, uint32_t, uint32_t, uint32_t) { return true; }
#endif

// Warp-aggregated append of `value` to queue[count++] for lanes with pred.
// Must be called by all 32 lanes of the warp.  Every queue holds up to
// pool_size entries.
PT_DI void q_push(const WfArgs& A, uint32_t* __restrict__ queue, uint32_t* count, uint32_t value, bool pred) {
    const unsigned mask = __ballot_sync(0xffffffffu, pred);
    if (mask == 0) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    const uint32_t at = base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
    if (pred && pt_check(A, at, A.pool_size, PT_CHECK_QUEUE_APPEND)) queue[at] = value;
}

// One 16-byte field of the pool's pairs (WfPool): element slot of a field
// is the first or second half of the slot's 32-byte pair.
template <typename T> struct PairField {
    T* p;
    PT_DI T& operator[](uint32_t slot) const { return p[2u * slot]; }
};
template <typename T> PT_DI PairField<T> first_of(float4* pair) { return PairField<T>{reinterpret_cast<T*>(pair)}; }
template <typename T> PT_DI PairField<T> second_of(float4* pair) {
    return PairField<T>{reinterpret_cast<T*>(pair) + 1};
}

struct PoolView {
    PairField<float4> s0, s1, s2, s3, s4, s5, s6, s7;  // see WfPool
    PairField<uint4> s8;
    PairField<float4> s9, h0, h1, m0, m1;
};

// The word in m1.z of a suspended march: bit 31 set, the SDF sign k
// (-1, 0, 1) + 1 in bits 26-27, points in bits 10-25 and the loop
// iterations in bits 0-9.  A ray fresh from intersection has 0 there.
PT_DI uint32_t march_word(float k, int points, int iter) {
    const uint32_t kc = (k > 0.0f) ? 2u : ((k < 0.0f) ? 0u : 1u);
    return 0x80000000u | (kc << 26) | ((uint32_t)min(points, 0xffff) << 10) | (uint32_t)iter;
}

PT_DI PoolView view(const WfArgs& A) {
    const WfPool& p = A.pool;
    return PoolView{first_of<float4>(p.s01), second_of<float4>(p.s01), first_of<float4>(p.s23),
                    second_of<float4>(p.s23), first_of<float4>(p.s49), first_of<float4>(p.s56),
                    second_of<float4>(p.s56), first_of<float4>(p.s78), second_of<uint4>(p.s78),
                    second_of<float4>(p.s49), first_of<float4>(p.h01), second_of<float4>(p.h01),
                    first_of<float4>(p.m01), second_of<float4>(p.m01)};
}

// s8.w packs the path's pass (its job-ring entry, 20 bits) with the
// object index of its sampled light (12 bits, signed): a ray's pass is read
// with its RNG word and flags in one load.
constexpr uint32_t kJobShift = 12;
static_assert(PT_MAX_SCENE_OBJECTS < 2048, "object indices must fit the 12-bit signed field of s8.w");
static_assert(kMaxJobRing <= (1u << (32 - kJobShift)), "job-ring entries must fit the 20-bit field of s8.w");
PT_DI uint32_t job_word(uint32_t job, int shObj) { return (job << kJobShift) | ((uint32_t)shObj & 0xFFFu); }
PT_DI uint32_t word_job(uint32_t w) { return w >> kJobShift; }
PT_DI int word_shobj(uint32_t w) { return (int)(w << 20) >> 20; }
PT_DI uint32_t slot_job(const PoolView& v, uint32_t slot) { return word_job(v.s8[slot].w); }

// SphereTracing (SC:779-860) with one SDF evaluation per loop iteration per
// lane.  A converged ray takes its six normal probes on its own lane
// (MP_NORMAL0..5), or waits in MP_NORMAL for the warp's normal pass
// (march_rays<true>).
enum MarchPhase { MP_EMPTY = 0, MP_SIGN = 1, MP_STEP = 2, MP_NORMAL0 = 3, MP_NORMAL5 = 8, MP_NORMAL = 9 };

// CalculateNumericalSDFNormals (SC:721-730) for the lanes of `pending` (rays
// converged at p): the six probes p +- h.xyy, h.yxy, h.yyx of up to five rays
// at once, one probe per lane, so the probes (near the surface, where an
// escape-time fractal runs its longest loops) fill the warp instead of one
// lane each beside rays that march far from it.  Measured on GB300: 11 %
// less march time on a 12-iteration mandelbulb, 2 % on the 4-iteration one,
// but 11 % more end to end on menger + terrain, whose evaluations cost the
// same everywhere and whose probes on the ray's own lane fill the rest of
// the round.  Returns the
// central-difference vector (+x - -x, +y - -y, +z - -z) to the lanes of
// `pending`.  Called by all 32 lanes with the same `pending`.
PT_DI float3 normal_probes(unsigned pending, const KScene* Sp, float3 p, uint32_t set1, int lane) {
    const float e = 1e-4f;
    float3 nv = f3(0.0f, 0.0f, 0.0f);
    while (pending) {
        // up to five rays, lowest lanes first (warp-uniform)
        unsigned take = 0, rest = pending;
        for (int c = 0; c < 5 && rest; c++) {
            take |= rest & (0u - rest);
            rest &= rest - 1u;
        }
        const int nray = __popc(take);
        const int r = lane / 6, j = lane - 6 * r;  // this lane: probe j of the r-th ray taken
        const bool probe = r < nray;
        unsigned m = take;  // drop the r lowest rays: the r-th ray is the lowest bit left
        for (int c = 0; c < r && c < 5; c++) m &= m - 1u;
        const int src = probe ? __ffs(m) - 1 : lane;
        const float px = __shfl_sync(0xffffffffu, p.x, src);
        const float py = __shfl_sync(0xffffffffu, p.y, src);
        const float pz = __shfl_sync(0xffffffffu, p.z, src);
        const uint32_t s1 = __shfl_sync(0xffffffffu, set1, src);
        const uint64_t sp = reinterpret_cast<uint64_t>(Sp);
        const uint32_t lo = __shfl_sync(0xffffffffu, (uint32_t)sp, src);
        const uint32_t hi = __shfl_sync(0xffffffffu, (uint32_t)(sp >> 32), src);
        float val = 0.0f;
        if (probe) {
            const KScene& S = *reinterpret_cast<const KScene*>((uint64_t)lo | ((uint64_t)hi << 32));
            const float ex = (j == 0) ? e : 0.0f, ey = (j == 2) ? e : 0.0f, ez = (j == 4) ? e : 0.0f;
            const float mx = (j == 1) ? e : 0.0f, my = (j == 3) ? e : 0.0f, mz = (j == 5) ? e : 0.0f;
            const float3 q = (j & 1) ? f3(px - mx, py - my, pz - mz) : f3(px + ex, py + ey, pz + ez);
            int esel = -1;
            val = scene_sdf_sel(S, q, s1, esel);
        }
        // Ray lane L collects the probes of its rank among `take`.
        const int base = 6 * __popc(take & ((1u << lane) - 1u));
        const float v0 = __shfl_sync(0xffffffffu, val, min(base + 0, 31));
        const float v1 = __shfl_sync(0xffffffffu, val, min(base + 1, 31));
        const float v2 = __shfl_sync(0xffffffffu, val, min(base + 2, 31));
        const float v3 = __shfl_sync(0xffffffffu, val, min(base + 3, 31));
        const float v4 = __shfl_sync(0xffffffffu, val, min(base + 4, 31));
        const float v5 = __shfl_sync(0xffffffffu, val, min(base + 5, 31));
        if ((take >> lane) & 1u) nv = f3(v0 - v1, v2 - v3, v4 - v5);
        pending &= ~take;
    }
    return nv;
}

// Warp-staged queue appends: lanes with pred add `value` to a per-warp
// buffer of 64 in shared memory (count warp-uniform); every 32 entries go to
// the queue with one atomic and one coalesced store.  Called by all 32 lanes.
PT_DI void stage_push(const WfArgs& A, uint32_t* buf, uint32_t& count, bool pred, uint32_t value, uint32_t* queue,
                      uint32_t* qcount, int lane) {
    const unsigned m = __ballot_sync(0xffffffffu, pred);
    if (!m) return;
    if (pred) buf[count + (uint32_t)__popc(m & ((1u << lane) - 1u))] = value;
    count += (uint32_t)__popc(m);  // < 64: it was < 32 before
    if (count < 32) return;
    __syncwarp();
    uint32_t b = 0;
    if (lane == 0) b = atomicAdd(qcount, 32u);
    b = __shfl_sync(0xffffffffu, b, 0);
    if (pt_check(A, b + (uint32_t)lane, A.pool_size, PT_CHECK_QUEUE_APPEND)) queue[b + (uint32_t)lane] = buf[lane];
    const uint32_t rest = count - 32;
    const uint32_t moved = ((uint32_t)lane < rest) ? buf[32 + lane] : 0u;
    __syncwarp();
    if ((uint32_t)lane < rest) buf[lane] = moved;
    __syncwarp();
    count = rest;
}

// Appends what stage_push still holds.  Called by all 32 lanes.
PT_DI void stage_flush(const WfArgs& A, uint32_t* buf, uint32_t count, uint32_t* queue, uint32_t* qcount, int lane) {
    __syncwarp();
    if (!count) return;
    uint32_t b = 0;
    if (lane == 0) b = atomicAdd(qcount, count);
    b = __shfl_sync(0xffffffffu, b, 0);
    if ((uint32_t)lane < count && pt_check(A, b + (uint32_t)lane, A.pool_size, PT_CHECK_QUEUE_APPEND))
        queue[b + (uint32_t)lane] = buf[lane];
}

// The march loop; WARP_NORMALS: normal probes in the warp's pass
// (normal_probes) instead of on each ray's lane.
template <bool WARP_NORMALS>
PT_DI void march_rays(const WfArgs& A) {
    WfCounters& C = *A.counters;
    const uint32_t cur = C.cur;
    const uint32_t n = C.n_march[cur];
    const uint32_t* __restrict__ qin = A.q_march[cur];
    const PoolView v = view(A);
    const PoolView& M = v;
    const int lane = threadIdx.x & 31;
    const int budget = A.march_budget;
    const int refill_min = A.refill_min;
    const int inner = A.march_inner;
    int steps = 0;
    // Draining only pays while the queue holds more rays than the grid has lanes.
    const bool many = n >= 2u * gridDim.x * blockDim.x;
    // Queue entries per claim: up to 32 while the queue is long, 1 near its end.
    const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
    const uint32_t chunk = max(1u, min(32u, n / (4u * nwarps)));
    uint32_t cbase = 0, cleft = 0;  // warp-uniform: unused entries of the warp's claim
    // Finished rays are staged per warp and kind and appended to the shade
    // queues 32 at a time.
    __shared__ uint32_t staged[kStageThreads / 32][2][64];
    uint32_t nstaged[2] = {0u, 0u};  // warp-uniform: primary hits, shadow results
    const int wib = (int)(threadIdx.x >> 5);

    uint32_t slot = 0;
    const KScene* Sp = nullptr;
    int phase = MP_EMPTY;
    bool exhausted = false;
    float3 org = f3(0.0f, 0.0f, 0.0f), dir = f3(0.0f, 0.0f, 1.0f), p = org;
    float t = 0.0f, insT = 0.0f, omega = 0.0f, prevR = 0.0f, hitdist = 0.0f, k = 0.0f, nplus = 0.0f;
    float3 nv = f3(0.0f, 0.0f, 0.0f);
    float2 tmm = make_float2(0.0f, 0.0f);
    uint32_t set1 = 0;
    int points = 0, iter = 0;
    bool xmarch = false;  // the ray's scene sets march limits (PT_EXT_MARCH; read from it where used)
    int hit_sel = -2;  // >= -1 once the lane's march converged (scene_sdf_material_hit)
    bool shadow_ray = false;
    const float omegaMax = kOmegaMax, omegaSpeed = 0.20f, e = 1e-4f;

    for (;;) {
        // Refill lanes that have no ray (warp-aggregated fetch), once at
        // least refill_min of them are idle or the warp has none left.
        // Queue entries come from a chunk the warp claimed with one atomic
        // (cbase, cleft: warp-uniform); a refill that needs more than the
        // chunk holds claims the next chunk.
        const bool need = (phase == MP_EMPTY) && !exhausted;
        const unsigned mneed = __ballot_sync(0xffffffffu, need);
        if (mneed && (__popc(mneed) >= refill_min || __ballot_sync(0xffffffffu, phase != MP_EMPTY) == 0)) {
            const uint32_t want = (uint32_t)__popc(mneed);
            const uint32_t from_old = min(want, cleft);  // entries left in the current chunk
            const uint32_t old_base = cbase;
            uint32_t nb = 0;
            if (want > from_old) {
                const uint32_t ncount = max(chunk, want - from_old);
                if (lane == 0) nb = atomicAdd(&C.march_cursor, ncount);
                nb = __shfl_sync(0xffffffffu, nb, 0);
                cbase = nb + (want - from_old);
                cleft = ncount - (want - from_old);
            } else {
                cbase += want;
                cleft -= want;
            }
            if (need) {
                const uint32_t rank = (uint32_t)__popc(mneed & ((1u << lane) - 1u));
                const uint32_t idx = (rank < from_old) ? old_base + rank : nb + (rank - from_old);
                if (idx < n && pt_check(A, qin[idx], A.pool_size, PT_CHECK_QUEUE_SLOT) &&
                    pt_check(A, slot_job(v, qin[idx]), A.job_cap, PT_CHECK_JOB)) {
                    slot = qin[idx];
                    const uint4 w8 = v.s8[slot];
                    Sp = A.jobs[word_job(w8.w)].scene;
                    const float4 o = v.s0[slot];
                    const uint32_t flags = w8.y;
                    shadow_ray = (flags & kShadowFlag) != 0;
                    const float4 d = shadow_ray ? v.s2[slot] : v.s1[slot];
                    org = f3(o.x, o.y, o.z);
                    dir = f3(d.x, d.y, d.z);
                    hitdist = v.h0[slot].x;
                    steps = 0;
                    hit_sel = -2;
                    // A ray from isect (flag bit clear: start with the sign
                    // probe) or one suspended by an earlier launch.
                    const float4 a0 = M.m0[slot], a1 = M.m1[slot];
                    const uint32_t saved = __float_as_uint(a1.z);
                    t = a0.x;
                    insT = a0.y;
                    omega = a0.z;
                    prevR = a0.w;
                    tmm = make_float2(a1.x, a1.y);
                    k = (float)(int)((saved >> 26) & 3u) - 1.0f;
                    set1 = __float_as_uint(a1.w);
                    iter = (int)(saved & 1023u);
                    points = (int)((saved >> 10) & 0xffffu);
                    xmarch = (Sp->ext.flags & PT_EXT_MARCH) != 0;
                    p = fma3s(dir, t, org);
                    phase = (saved & 0x80000000u) ? MP_STEP : MP_SIGN;
                } else if (idx >= n) {
                    exhausted = true;
                }
            }
        }
        const unsigned live = __ballot_sync(0xffffffffu, phase != MP_EMPTY);
        if (live == 0) break;
        // Once the queue is drained, a warp with few rays left would run on
        // with most lanes idle: its marching rays save their state and
        // continue in full warps next iteration instead.
        const bool drain = many && __ballot_sync(0xffffffffu, exhausted) != 0 && __popc(live) < A.drain_lanes;

        // A.march_inner SDF evaluations per lane before the warp refills,
        // shades finished hits and appends to the queues again: the warp
        // pays for those once per several evaluations, and a lane whose ray
        // finishes or is suspended on the way idles until then.
        bool finished = false, hit = false, suspend = false;
#pragma unroll 1
        for (int sub = 0; sub < inner; sub++) {
            // One SDF evaluation.
            const bool evalLane = (phase >= MP_SIGN && phase <= MP_NORMAL5) && !finished && !suspend;
            if (sub > 0 && __ballot_sync(0xffffffffu, evalLane) == 0) break;
            float3 q = p;
            if (phase == MP_SIGN) q = org;
            if (!WARP_NORMALS && phase >= MP_NORMAL0 && phase <= MP_NORMAL5) {
                // CalculateNumericalSDFNormals (SC:721-730): p +- h.xyy, h.yxy, h.yyx
                const int j = phase - MP_NORMAL0;
                const float ex = (j == 0) ? e : 0.0f, ey = (j == 2) ? e : 0.0f, ez = (j == 4) ? e : 0.0f;
                const float mx = (j == 1) ? e : 0.0f, my = (j == 3) ? e : 0.0f, mz = (j == 5) ? e : 0.0f;
                q = (j & 1) ? f3(p.x - mx, p.y - my, p.z - mz) : f3(p.x + ex, p.y + ey, p.z + ez);
            }
            float val = 0.0f;
            int esel = -1;
            if (evalLane) val = scene_sdf_sel(*Sp, q, set1, esel);
            if (!evalLane) continue;
            if (phase == MP_SIGN) {
                k = sign_glsl(val);
                phase = MP_STEP;
            } else if (phase == MP_STEP) {
                const float radius = val;
                bool exitLoop = false;
                if (xmarch && t > Sp->ext.march_max_distance) {
                    finished = true;  // past the distance cap: no SDF hit
                } else if (insT > (fabsf(prevR) + fabsf(radius))) {
                    t -= insT;
                    omega = 1.0f;
                    insT = prevR * omega * k;
                    t += insT;
                    p = fma3s(dir, t, org);
                } else if (fabsf(radius) < (xmarch ? Sp->ext.march_epsilon : 1e-4f)) {
                    exitLoop = true;
                    hit_sel = esel;
                } else {
                    if (t > tmm.y) {
                        points += 1;
                    } else {
                        points = 0;
                    }
                    bool researched = false;
                    if (points >= 2) {
                        t = tmm.y + 1e-3f;
                        tmm = make_float2(PT_MAXDIST, PT_MAXDIST);
                        const float3 invdir = f3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
                        if (search_sdf(*Sp, fma3s(dir, t, org), invdir, tmm, set1)) {
                            tmm.x += t;
                            tmm.y += t;
                            t = fmaxf(tmm.x, t);
                            p = fma3s(dir, t, org);
                            researched = true;
                        } else {
                            finished = true;  // left every SDF box: no SDF hit
                        }
                    }
                    if (!finished && !researched) {
                        insT = radius * omega * k;
                        t += insT;
                        p = fma3s(dir, t, org);
                        const float omegaSpeedFactor = fminf(radius / prevR, 0.99f);
                        omega += omegaSpeed * (fminf(1.0f / (1.0f - omegaSpeedFactor), omegaMax) - omega);
                        prevR = radius;
                    }
                }
                if (!finished && !exitLoop) {
                    iter++;
                    if (iter >= (xmarch ? Sp->ext.march_max_steps : 512)) exitLoop = true;
                }
                if (exitLoop) {
                    if (t < hitdist) {
                        p = fma3s(dir, t, org);
                        phase = WARP_NORMALS ? MP_NORMAL : MP_NORMAL0;
                    } else {
                        finished = true;
                    }
                } else if (!finished && (++steps >= budget || (drain && steps >= kDrainMinSteps))) {
                    // out of budget for this launch: save the state, continue next iteration
                    M.m0[slot] = make_float4(t, insT, omega, prevR);
                    M.m1[slot] = make_float4(tmm.x, tmm.y, __uint_as_float(march_word(k, points, iter)),
                                             __uint_as_float(set1));
                    suspend = true;
                }
            } else if (!WARP_NORMALS && phase >= MP_NORMAL0 && phase <= MP_NORMAL5) {
                const int j = phase - MP_NORMAL0;
                if ((j & 1) == 0) {
                    nplus = val;
                } else {
                    const float dv = nplus - val;
                    if (j == 1) nv.x = dv;
                    else if (j == 3) nv.y = dv;
                    else nv.z = dv;
                }
                phase++;
                if (phase > MP_NORMAL5) {
                    hit = true;
                    finished = true;
                }
            }
        }

        if constexpr (WARP_NORMALS) {
            // The normals of this round's converged rays, six probes a ray
            // across the warp.
            const unsigned pending = __ballot_sync(0xffffffffu, phase == MP_NORMAL);
            if (pending) {
                const float3 nw = normal_probes(pending, Sp, p, set1, lane);
                if (phase == MP_NORMAL) {
                    hit = true;
                    finished = true;
                    const float3 nrm = normalize3(nw);
                    const float mat = scene_sdf_material_hit(*Sp, p, set1, hit_sel);
                    v.h0[slot] = make_float4(t - 1e-3f, mat, -1.0f, __int_as_float(-2));
                    v.h1[slot] = make_float4(nrm.x, nrm.y, nrm.z, 0.0f);
                }
            }
        } else if (finished && hit) {
            const float3 nrm = normalize3(nv);
            const float mat = scene_sdf_material_hit(*Sp, p, set1, hit_sel);
            v.h0[slot] = make_float4(t - 1e-3f, mat, -1.0f, __int_as_float(-2));
            v.h1[slot] = make_float4(nrm.x, nrm.y, nrm.z, 0.0f);
        }
        stage_push(A, staged[wib][0], nstaged[0], finished && !shadow_ray, slot, A.q_shade[cur], &C.n_shade[cur],
                   lane);
        stage_push(A, staged[wib][1], nstaged[1], finished && shadow_ray, slot, A.q_shadow[cur], &C.n_shadow[cur],
                   lane);
        q_push(A, A.q_march[cur ^ 1u], &C.n_march[cur ^ 1u], slot, suspend);
        if (finished || suspend) phase = MP_EMPTY;
    }
    // The staged remainders.
    stage_flush(A, staged[wib][0], nstaged[0], A.q_shade[cur], &C.n_shade[cur], lane);
    stage_flush(A, staged[wib][1], nstaged[1], A.q_shadow[cur], &C.n_shadow[cur], lane);
}

#if defined(PT_JIT_USER_SDF)
// Run-time compiled snippets: the warp's normal pass (escape-time fractals
// are the usual reason to write one, and their cost is not known here).
__global__ void PT_MARCH_BOUNDS wf_march(const __grid_constant__ WfArgs A) { march_rays<true>(A); }
#else
// The shipped plug-ins: normals on each ray's lane (menger, terrain and blob
// cost the same everywhere), or in the warp's pass when a mandelbulb is in
// the dispatch (the host picks the kernel).
__global__ void PT_MARCH_BOUNDS wf_march(const __grid_constant__ WfArgs A) { march_rays<false>(A); }
__global__ void PT_MARCH_BOUNDS wf_march_warp_normals(const __grid_constant__ WfArgs A) { march_rays<true>(A); }
#endif

}  // namespace
