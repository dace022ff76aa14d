// pt_megakernel.cu — the plain per-pixel spectral path tracer for sm_103a.
//
// One thread owns one pixel and traces its samplesPerFrame camera paths in
// order, like main()/Rendering() in src/shader.comp (SC:1509-1533), so the
// per-pixel sum and the running mean are formed in the reference's order.
// Inside the thread the path is a small state machine with ONE call site of
// intersect_all(): a primary ray, then (when next-event estimation needs it)
// the shadow ray of the same bounce, then the next bounce or the next sample.
// Lanes of a warp that are at different bounces, samples or ray kinds still
// execute the scene intersection and SDF march together, instead of
// splitting into a primary-ray pass and a shadow-ray pass.
#include <cuda_runtime.h>

#include "pt_geometry.cuh"
#include "pt_megakernel.h"

namespace {

// PCG32 hash, SC:937-946.
PT_DI uint32_t pcg32(uint32_t seed) {
    const uint32_t state = seed * 747796405u + 2891336453u;
    const uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
// float(seed) / float(0xFFFFFFFFu): round-to-nearest conversion, divisor 2^32.
PT_DI float rnd(uint32_t& seed) {
    seed = pcg32(seed);
    return __uint2float_rn(seed) / 4294967296.0f;
}

// WaveToXYZ, SC:129-140, from the CIE table in global memory.
PT_DI float cie_at(const float* __restrict__ cie, int i) {
    return ((unsigned)i < (unsigned)PT_CIE_TABLE_SIZE) ? __ldg(cie + i) : 0.0f;
}
PT_DI float3 wave_to_xyz(const float* __restrict__ cie, float wave) {
    float3 r = f3(0.0f, 0.0f, 0.0f);
    if ((wave >= 360.0f) && (wave <= 800.0f)) {
        const int i3 = 3 * (int)(floorf(wave) - 360.0f);
        const float a = wave - floorf(wave);
        r = f3(mix_glsl(cie_at(cie, i3), cie_at(cie, i3 + 3), a), mix_glsl(cie_at(cie, i3 + 1), cie_at(cie, i3 + 4), a),
               mix_glsl(cie_at(cie, i3 + 2), cie_at(cie, i3 + 5), a));
    }
    return r;
}

// SpectralPowerDistribution / EvaluateBRDF, SC:1030-1038, SC:1075-1080.
PT_DI float4 evaluate_brdf(float4 l, float peak, float sigma, float invertf) {
    const float den = 2.0f * sigma * sigma;
    const float4 x = f4((l.x - peak) / den, (l.y - peak) / den, (l.z - peak) / den, (l.w - peak) / den);
    const float4 r = f4(ptm_expf(-x.x * x.x), ptm_expf(-x.y * x.y), ptm_expf(-x.z * x.z), ptm_expf(-x.w * x.w));
    const float a = (float)(int)invertf;
    const float4 s = f4(mix_glsl(r.x, 1.0f - r.x, a), mix_glsl(r.y, 1.0f - r.y, a), mix_glsl(r.z, 1.0f - r.z, a),
                        mix_glsl(r.w, 1.0f - r.w, a));
    return s / PT_PI;
}

// BlackBodyRadiation / Emit, SC:1040-1055.
PT_DI float blackbody(float l, float T) {
    return (1.1910429724e-16f * ptm_powf(l, -5.0f)) / (ptm_expf(0.014387768775f / (l * T)) - 1.0f);
}
PT_DI float4 emit(float4 l, float temperature_in, float luminosity) {
    const float T = fmaxf(temperature_in, 0.0f);
    const float4 lm = l * 1e-9f;
    const float peak = 4.0956746759e-6f * ptm_powf(T, 5.0f);
    const float4 e = f4(blackbody(lm.x, T) / peak, blackbody(lm.y, T) / peak, blackbody(lm.z, T) / peak,
                        blackbody(lm.w, T) / peak);
    return e * fmaxf(luminosity, 0.0f);
}

// RefractiveIndexBK7Glass, SC:1064-1073.
PT_DI float bk7_index(float l) {
    l *= 1e-3f;
    const float l2 = l * l;
    float n2 = 1.0f;
    n2 += (1.03961212f * l2) / (l2 - 6.00069867e-3f);
    n2 += (0.231792344f * l2) / (l2 - 2.00179144e-2f);
    n2 += (1.01046945f * l2) / (l2 - 1.03560653e2f);
    return sqrtf(n2);
}

// OrthonormalBasis + ToWorld, SC:1093-1119.
PT_DI float3 to_world(float3 v, float3 n) {
    float3 b1 = f3(0.0f, -1.0f, 0.0f);
    float3 b2 = f3(-1.0f, 0.0f, 0.0f);
    if (n.z >= -0.9999999f) {
        const float a = 1.0f / (1.0f + n.z);
        const float b = -n.x * n.y * a;
        b1 = f3(1.0f - (n.x * n.x * a), b, -n.x);
        b2 = f3(b, 1.0f - (n.y * n.y * a), -n.y);
    }
    return b1 * v.x + b2 * v.y + n * v.z;
}

// GetMaterialMix, SC:237-249.
PT_DI float3 material_mix(const KScene& S, float materialID) {
    const int i1 = 3 * (int)floorf(materialID);
    const int i2 = 3 * (int)ceilf(materialID);
    const float x = materialID - floorf(materialID);
    return f3(mix_glsl(s_mat(S, i1), s_mat(S, i2), x), mix_glsl(s_mat(S, i1 + 1), s_mat(S, i2 + 1), x),
              mix_glsl(s_mat(S, i1 + 2), s_mat(S, i2 + 2), x));
}
// UnpackLight via GetLightMix, SC:224-235, SC:251-254.
PT_DI float2 light_mix(const KScene& S, float lightID) {
    const int index = (int)lightID;
    if (index == -1) return make_float2(5500.0f, 0.0f);
    return make_float2(s_light(S, 2 * index), s_light(S, 2 * index + 1));
}

// SampleRandomLightSource, SC:1225-1285, quirks included: the lens branch
// compares with the box count (SC:1264) and the cyclide branch with the lens
// count (SC:1275).  Object reads are guarded: these indices come from data.
PT_DI int sample_random_light(const KScene& S, uint32_t& seed, float& boundingRadius, float3& pos, float& lightID,
                              int& pick) {
    const int randomLight = (int)floorf(rnd(seed) * S.numObjects[6]);
    pick = randomLight;
    const int result = (int)s_lightid(S, randomLight);
    int L = result;
    int offset = 0;
    const int* n = S.meta.n;
    if (L < n[0]) {
        const int b = 6 * L;
        boundingRadius = s_obj(S, b + 3);
        pos = f3(s_obj(S, b), s_obj(S, b + 1), s_obj(S, b + 2));
        lightID = (float)((int)s_obj(S, b + 5) - 1);
        return result;
    }
    L -= n[0];
    offset += 6 * n[0];
    if (L < n[1]) {
        const int b = 5 * L + offset;
        boundingRadius = 1e5f;
        pos = f3(s_obj(S, b), s_obj(S, b + 1), s_obj(S, b + 2));
        lightID = (float)((int)s_obj(S, b + 4) - 1);
        return result;
    }
    L -= n[1];
    offset += 5 * n[1];
    if (L < n[2]) {
        const int b = 11 * L + offset;
        boundingRadius = 0.5f * length3(f3(s_obj(S, b + 6), s_obj(S, b + 7), s_obj(S, b + 8)));
        pos = f3(s_obj(S, b), s_obj(S, b + 1), s_obj(S, b + 2));
        lightID = (float)((int)s_obj(S, b + 10) - 1);
        return result;
    }
    L -= n[2];
    offset += 11 * n[2];
    if (L < n[2]) {
        const int b = 12 * L + offset;
        const float r = s_obj(S, b + 6), th = s_obj(S, b + 8);
        boundingRadius = sqrtf((r * r) + (0.25f * th * th));
        pos = f3(s_obj(S, b), s_obj(S, b + 1), s_obj(S, b + 2));
        lightID = (float)((int)s_obj(S, b + 11) - 1);
        return result;
    }
    L -= n[3];
    offset += 12 * n[3];
    if (L < n[3]) {
        const int b = 16 * L + offset;
        boundingRadius = sqrtf(s_obj(S, b + 13));
        pos = f3(s_obj(S, b), s_obj(S, b + 1), s_obj(S, b + 2));
        lightID = (float)((int)s_obj(S, b + 15) - 1);
        return result;
    }
    return 0;
}

// Per-block camera: the camera basis and the camera lens depend only on the
// push constants, so one thread derives them per block (SC:1456, SC:1409-1418).
struct CamShared {
    m3 cam;
    m3 lensRot;
    float3 lensPos;
};

template <bool TRACE>
__global__ void __launch_bounds__(PT_MK_THREADS) megakernel(const __grid_constant__ KParams P) {
    const KScene& S = P.s;
    const pt_push& pc = P.pc;
    __shared__ CamShared camS;
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        const m3 cam = rotation_matrix(f3(pc.cameraAngle[0], pc.cameraAngle[1], 0.0f));
        const float3 camPos = f3(pc.cameraPosX, pc.cameraPosY, pc.cameraPosZ);
        const float3 fwd = f3(cam.c0.z, cam.c1.z, cam.c2.z);
        camS.cam = cam;
        camS.lensRot = rotation_matrix(f3(0.0f, 90.0f - pc.cameraAngle[1], pc.cameraAngle[0]));
        camS.lensPos = camPos + fwd * pc.lensDistance;
    }
    __syncthreads();

    const int W = pc.resolution[0], H = pc.resolution[1];
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= W || y >= H) return;  // SC:1526 uses '>'; the extra row/column would write out of bounds

    const uint32_t xx = (uint32_t)x;
    const uint32_t yy = (uint32_t)H - (uint32_t)y;  // SC:1510
    const float uvx = (2.0f * (float)xx - (float)W) / (float)H;
    const float uvy = (2.0f * (float)yy - (float)H) / (float)H;
    const int spf = pc.samplesPerFrame;
    const int depth = pc.pathLength;
    const float numLights = S.numObjects[6];
    const size_t pix = (size_t)y * (size_t)W + (size_t)x;

    float3 sum = f3(0.0f, 0.0f, 0.0f);
    int k = 0;

    // Path state.
    uint32_t seed = 0;
    float3 org = f3(0.0f, 0.0f, 0.0f), dir = f3(0.0f, 0.0f, 1.0f);
    float4 l = f4s(0.0f), radiance = f4s(0.0f), rr = f4s(1.0f);
    float mis = 1.0f;
    int bounce = 0;
    bool active = false;
    // State of the bounce between its primary hit and its shadow ray.
    bool shadow = false;
    float3 nrm = f3(0.0f, 0.0f, 0.0f), shDir = f3(0.0f, 0.0f, 1.0f);
    float4 brdf = f4s(0.0f);
    float brdfPdf = 0.0f, lightPdf = 0.0f, cosL = 0.0f, shLightID = -1.0f;
    int shObj = 0;
    uint32_t ev = 0;

    for (;;) {
        if (!active) {
            // Finish sample k-1 (SC:1477-1489) and start sample k (SC:1446-1476).
            if (k > 0) {
                const float3 wx = wave_to_xyz(P.cie, l.x), wy = wave_to_xyz(P.cie, l.y);
                const float3 wz = wave_to_xyz(P.cie, l.z), ww = wave_to_xyz(P.cie, l.w);
                float3 color = (((wx * radiance.x + wy * radiance.y) + wz * radiance.z) + ww * radiance.w) *
                               (720.0f - 390.0f) * 0.25f;
                if (color.x != color.x || color.y != color.y || color.z != color.z) color = f3(0.0f, 0.0f, 0.0f);
                if (TRACE) {
                    const size_t p = pix * (size_t)spf + (size_t)(k - 1);
                    if (P.trace.nevents) P.trace.nevents[p] = (uint32_t)bounce;
                    if (P.trace.colors) {
                        P.trace.colors[3 * p] = color.x;
                        P.trace.colors[3 * p + 1] = color.y;
                        P.trace.colors[3 * p + 2] = color.z;
                    }
                }
                sum = sum + color;
            }
            if (k >= spf) break;
            // GenerateSeed SC:948-958, SSAA SC:1449, camera SC:1455-1465.
            seed = pcg32((uint32_t)(pc.frame - spf + k)) + (xx + (uint32_t)W * yy);
            const float jx = 2.0f * rnd(seed) - 0.5f;
            const float jy = 2.0f * rnd(seed) - 0.5f;
            const float sc = -pc.cameraSize * 0.5f;
            const float u = (uvx + jx / (float)W) * sc;
            const float v = (uvy + jy / (float)H) * sc;
            const float3 camPos = f3(pc.cameraPosX, pc.cameraPosY, pc.cameraPosZ);
            org = camPos + mul_vm(f3(u, v, 0.0f), camS.cam);
            const float rx = rnd(seed);
            const float ry = rnd(seed);
            const float phi = 2.0f * PT_PI * ry;
            const float dd = sqrtf(rx);
            const float ha = 0.5f * pc.apertureSize;
            float sp, cp;
            ptm_sincosf(phi, &sp, &cp);
            const float3 poa = camPos + mul_vm(f3(ha * (dd * cp), ha * (dd * sp), pc.apertureDist), camS.cam);
            dir = normalize3(poa - org);
            // SampleHeroWavelength SC:960-963, TracePathLens SC:1409-1444.
            const float lh = mix_glsl(360.0f, 800.0f, rnd(seed));
            {
                LensGeom cl;
                cl.pos = camS.lensPos;
                cl.rot = camS.lensRot;
                cl.radius = pc.lensRadius;
                cl.focal = pc.lensFocalLength;
                cl.thickness = pc.lensThickness;
                cl.converging = true;
                float lam = lh;
#pragma unroll 1
                for (int i = 0; i < 2; i++) {
                    Hit h;
                    h.hitdist = 1e6f;
                    h.normal = f3(0.0f, 0.0f, 0.0f);
                    h.materialID = 0.0f;
                    h.lightID = -1.0f;
                    int isOutside = 1;
                    lens_intersect(org, dir, cl, 0.0f, -1.0f, h, isOutside);
                    float n1, n2;
                    if (isOutside == 1) {
                        n1 = 1.0f;
                        n2 = bk7_index(lam);
                    } else {
                        n1 = bk7_index(lam);
                        n2 = 1.0f;
                    }
                    const float n12 = n1 / n2;
                    lam = lam * n12;
                    org = fma3s(dir, h.hitdist, org);
                    dir = refract3(dir, h.normal, n12);
                }
            }
            // SampleWavelengths SC:971-974.
            const float base = lh - 390.0f;
            l = f4(390.0f + mod_glsl(base + 82.5f, 330.0f), 390.0f + mod_glsl(base + 165.0f, 330.0f),
                   390.0f + mod_glsl(base + 247.5f, 330.0f), 390.0f + mod_glsl(base + 330.0f, 330.0f));
            radiance = f4s(0.0f);
            rr = f4s(1.0f);
            mis = 1.0f;
            bounce = 0;
            shadow = false;
            k++;
            active = depth > 0;
            continue;
        }

        // ---- the single scene intersection of the loop ----
        Hit h;
        h.hitdist = PT_MAXDIST;
        h.normal = f3(0.0f, 0.0f, 0.0f);
        h.materialID = 0.0f;
        h.lightID = -1.0f;
        int objectID = -1;
        intersect_all(S, org, shadow ? shDir : dir, h, objectID);

        bool finishBounce = false;
        if (!shadow) {
            // TraceRay, SC:1345-1391.
            ev = PT_EV_VALID;
            if (h.hitdist < PT_MAXDIST) {
                if (TRACE) ev |= (objectID == -2) ? PT_EV_HIT_SDF : ((uint32_t)objectID & PT_EV_HIT_MASK);
                const float2 lt = light_mix(S, h.lightID);
                if (lt.y > 0.0f) {
                    radiance = radiance + (emit(l, lt.x, lt.y) * rr) * mis;
                    if (TRACE) ev |= PT_EV_EMITTER;
                    active = false;
                } else {
                    const float3 mat = material_mix(S, h.materialID);
                    brdf = evaluate_brdf(l, mat.x, mat.y, mat.z);
                    nrm = h.normal;
                    org = fma3s(dir, h.hitdist, org);
                    {  // SampleBRDF: cosine direction via the unit sphere, SC:984-1003.
                        const float rx = rnd(seed);
                        const float ry = rnd(seed);
                        const float phi = 2.0f * PT_PI * ry;
                        const float sinTheta = 2.0f * rx - 1.0f;
                        const float cosTheta = sqrtf(__fmaf_rn(-sinTheta, sinTheta, 1.0f));
                        float sp, cp;
                        ptm_sincosf(phi, &sp, &cp);
                        dir = normalize3(nrm + f3(cp * cosTheta, sp * cosTheta, sinTheta));
                    }
                    brdfPdf = dot3(dir, nrm) / PT_PI;
                    // SampleLightSource, SC:1298-1343.
                    int pick = 0;
                    uint32_t shadowState = 0;
                    if (numLights > 0.0f) {
                        float boundingRadius = 0.0f;
                        float3 lightPos = f3(0.0f, 0.0f, 0.0f);
                        shLightID = -1.0f;
                        shObj = sample_random_light(S, seed, boundingRadius, lightPos, shLightID, pick);
                        const float invLightDistance = 1.0f / length3(lightPos - org);
                        const float3 lightDir = (lightPos - org) * invLightDistance;
                        const float sinthetaMax = fminf(boundingRadius * invLightDistance, 1.0f);
                        const float costhetaMax = sqrtf(1.0f - sinthetaMax * sinthetaMax);
                        {  // SampleCosineUnitCone, SC:1012-1023.
                            const float rx = rnd(seed);
                            const float ry = rnd(seed);
                            const float cosAlphaMax = 2.0f * costhetaMax * costhetaMax - 1.0f;
                            const float phi = 2.0f * PT_PI * ry;
                            const float cosTheta = (1.0f - cosAlphaMax) * rx + cosAlphaMax;
                            const float sinTheta = sqrtf(__fmaf_rn(-cosTheta, cosTheta, 1.0f));
                            float sp, cp;
                            ptm_sincosf(phi, &sp, &cp);
                            shDir = to_world(normalize3(f3(cp * sinTheta, sp * sinTheta, cosTheta + 1.0f)), lightDir);
                        }
                        lightPdf = 1.0f / numLights;
                        lightPdf *= dot3(shDir, lightDir) / (PT_PI * (1.0f - costhetaMax * costhetaMax));
                        mis = brdfPdf * brdfPdf / (brdfPdf * brdfPdf + lightPdf * lightPdf);
                        cosL = dot3(shDir, nrm);
                        const float deathProbability = 1.25f * fmaxf(mis - 0.2f, 0.0f);
                        if (cosL >= 0.0f) {
                            if (rnd(seed) > deathProbability) {
                                shadow = true;  // trace the shadow ray next iteration
                            } else {
                                mis = 1.0f;
                                shadowState = 1;
                            }
                        }
                    } else {
                        mis = brdfPdf * brdfPdf / (brdfPdf * brdfPdf + 0.0f * 0.0f);
                    }
                    if (TRACE) ev |= ((uint32_t)(pick & 0x7F) << PT_EV_LIGHT_SHIFT) | (shadowState << PT_EV_SHADOW_SHIFT);
                    if (!shadow) {
                        radiance = radiance + f4s(0.0f);
                        finishBounce = true;
                    }
                }
            } else {
                if (TRACE) ev |= PT_EV_HIT_MISS;
                radiance = radiance + f4s(0.0f);
                active = false;
            }
        } else {
            // LightSourceVisibilityCheck result, SC:1121-1223, and the NEE term.
            shadow = false;
            const int obj = (objectID == -2) ? -1 : objectID;
            float4 contrib = f4s(0.0f);
            if (obj == shObj) {
                const float2 lt = light_mix(S, shLightID);
                const float4 rrl = rr * ((brdf * cosL) / lightPdf);
                contrib = (emit(l, lt.x, lt.y) * rrl) * (1.0f - mis);
                if (TRACE) ev |= 3u << PT_EV_SHADOW_SHIFT;
            } else {
                if (TRACE) ev |= 2u << PT_EV_SHADOW_SHIFT;
            }
            radiance = radiance + contrib;
            finishBounce = true;
        }

        if (finishBounce) {
            // BRDF throughput and Russian roulette, SC:1373-1385.
            const float costheta = dot3(dir, nrm);
            rr = rr * ((brdf * costheta) / brdfPdf);
            const float rp = fminf(fmaxf(fmaxf(rr.x, fmaxf(rr.y, fmaxf(rr.z, rr.w))), 0.0f), 0.99f);
            if (rnd(seed) > rp) {
                if (TRACE) ev |= PT_EV_RR_KILL;
                active = false;
            } else {
                rr = rr * (1.0f / rp);
            }
        }
        if (!shadow) {
            // The bounce is complete: record it and stop at pathLength (SC:1400).
            if (TRACE) {
                const size_t p = pix * (size_t)spf + (size_t)(k - 1);
                if (P.trace.events && bounce < P.trace.cap) P.trace.events[p * (size_t)P.trace.cap + bounce] = ev;
            }
            bounce++;
            if (bounce >= depth) active = false;
        }
    }

    // Rendering + Accumulate, SC:1513-1520, SC:1492-1507.
    const float fs = (float)spf;
    float3 out = f3(sum.x / fs, sum.y / fs, sum.z / fs);
    out = out * (pc.apertureSize * pc.apertureSize * (float)pc.ISO);
    const float4 old = P.accum[pix];
    const float3 in = f3(old.x, old.y, old.z);
    if ((pc.currentSamples == pc.samplesPerFrame) && (pc.frame > pc.samplesPerFrame)) {
        const float w = ptm_powf(2.0f, -8.0f / (pc.FPS * pc.persistence));
        out = out * (1.0f - w) + in * w;
    } else {
        const int unitSamples = pc.currentSamples / pc.samplesPerFrame;
        const float us = (float)unitSamples;
        const float3 t = in * (float)(unitSamples - 1) + out;
        out = f3(t.x / us, t.y / us, t.z / us);
    }
    P.accum[pix] = make_float4(out.x, out.y, out.z, 1.0f);
}

// Per-upload derivation of the rotation matrices of boxes, lenses and cyclides.
__global__ void rotation_setup_kernel(const __grid_constant__ KScene S, float* __restrict__ out) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= S.meta.total_objects) return;
    const int* n = S.meta.n;
    int base = -1;
    if (g >= n[0] + n[1]) {
        int i = g - n[0] - n[1];
        if (i < n[2]) {
            base = S.meta.offset[2] + 11 * i;
        } else if ((i -= n[2]) < n[3]) {
            base = S.meta.offset[3] + 12 * i;
        } else {
            i -= n[3];
            base = S.meta.offset[4] + 16 * i;
        }
    }
    float r[9] = {1.0f, 0.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.0f, 1.0f};
    if (base >= 0) {
        const m3 m = rotation_matrix(f3(S.objects[base + 3], S.objects[base + 4], S.objects[base + 5]));
        r[0] = m.c0.x; r[1] = m.c0.y; r[2] = m.c0.z;
        r[3] = m.c1.x; r[4] = m.c1.y; r[5] = m.c1.z;
        r[6] = m.c2.x; r[7] = m.c2.y; r[8] = m.c2.z;
    }
#pragma unroll
    for (int j = 0; j < 9; j++) out[9 * g + j] = r[j];
}

}  // namespace

namespace {
__global__ void mathf_eval_kernel(int fn, const float* __restrict__ x, const float* __restrict__ y,
                                  float* __restrict__ out, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float r;
    switch (fn) {
        case 0: r = ptm_sinf(x[i]); break;
        case 1: r = ptm_cosf(x[i]); break;
        case 2: r = ptm_expf(x[i]); break;
        case 3: r = ptm_logf(x[i]); break;
        case 4: r = ptm_powf(x[i], y[i]); break;
        default: r = ptm_acosf(x[i]); break;
    }
    out[i] = r;
}
}  // namespace

cudaError_t ptk_mathf_eval(int fn, const float* x, const float* y, float* out, int n, cudaStream_t stream) {
    if (n <= 0) return cudaSuccess;
    mathf_eval_kernel<<<(n + 255) / 256, 256, 0, stream>>>(fn, x, y, out, n);
    return cudaGetLastError();
}

cudaError_t ptk_rotation_setup(const KScene* scene, float* d_out, cudaStream_t stream) {
    const int n = scene->meta.total_objects;
    if (n <= 0) return cudaSuccess;
    rotation_setup_kernel<<<(n + 127) / 128, 128, 0, stream>>>(*scene, d_out);
    return cudaGetLastError();
}

cudaError_t ptk_launch_megakernel(const KParams* params, bool trace, cudaStream_t stream) {
    const int W = params->pc.resolution[0], H = params->pc.resolution[1];
    const dim3 block(PT_MK_BLOCK_X, PT_MK_BLOCK_Y);
    const dim3 grid((W + PT_MK_BLOCK_X - 1) / PT_MK_BLOCK_X, (H + PT_MK_BLOCK_Y - 1) / PT_MK_BLOCK_Y);
    if (trace) {
        megakernel<true><<<grid, block, 0, stream>>>(*params);
    } else {
        megakernel<false><<<grid, block, 0, stream>>>(*params);
    }
    return cudaGetLastError();
}
