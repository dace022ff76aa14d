// pt_path.cuh — one path's arithmetic, shared by both engines.
//
// The megakernel keeps a PathState in registers and loops; the wavefront
// renderer keeps it in a structure-of-arrays pool in HBM between stage
// kernels.  Both call these functions, in the same order, so a path computes
// the same bits in either engine (and in the CPU restatement).
#pragma once

#include "pt_geometry.cuh"

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
// One lobe of the multi-lobe Gaussian CIE fit (Wyman, Sloan and Shirley
// 2013): a Gaussian with a different width on each side of its peak.
PT_DI float cmf_lobe(float x, float mu, float s1, float s2) {
    const float t = (x - mu) / ((x < mu) ? s1 : s2);
    return ptm_expf(-0.5f * t * t);
}
// The fit itself at wavelength `wave` (nm), for PT_EXT_ANALYTIC_CMF.
PT_DI float3 cmf_analytic(float wave) {
    const float x = (1.056f * cmf_lobe(wave, 599.8f, 37.9f, 31.0f) + 0.362f * cmf_lobe(wave, 442.0f, 16.0f, 26.7f)) -
                    0.065f * cmf_lobe(wave, 501.1f, 20.4f, 26.2f);
    const float y = 0.821f * cmf_lobe(wave, 568.8f, 46.9f, 40.5f) + 0.286f * cmf_lobe(wave, 530.9f, 16.3f, 31.1f);
    const float z = 1.217f * cmf_lobe(wave, 437.0f, 11.8f, 36.0f) + 0.681f * cmf_lobe(wave, 459.0f, 26.0f, 13.8f);
    return f3(x, y, z);
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
// pow(l, -5) as ptm_powf computes it, 1 / l^5 by binary powering (l > 0).
PT_DI float blackbody(float l, float T) {
    return (1.1910429724e-16f * (1.0f / pow_pos_int<5>(l))) / (ptm_expf(0.014387768775f / (l * T)) - 1.0f);
}
PT_DI float4 emit(float4 l, float temperature_in, float luminosity) {
    const float T = fmaxf(temperature_in, 0.0f);
    const float4 lm = l * 1e-9f;
    const float peak = 4.0956746759e-6f * pow_pos_int<5>(T);  // T >= 0
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


PT_DI CamInfo make_camera(const pt_push& pc) {
    CamInfo c;
    c.cam = rotation_matrix(f3(pc.cameraAngle[0], pc.cameraAngle[1], 0.0f));
    const float3 camPos = f3(pc.cameraPosX, pc.cameraPosY, pc.cameraPosZ);
    const float3 fwd = f3(c.cam.c0.z, c.cam.c1.z, c.cam.c2.z);
    c.lensRot = rotation_matrix(f3(0.0f, 90.0f - pc.cameraAngle[1], pc.cameraAngle[0]));
    c.lensPos = camPos + fwd * pc.lensDistance;
    return c;
}

// The state of one camera path between scene intersections.
struct PathState {
    float3 org, dir;         // path ray (after a non-emissive hit: the new origin and the BRDF direction)
    float4 l, radiance, rr;  // wavelengths, accumulated radiance, throughput
    float mis;               // MISBRDFWeight
    uint32_t seed;
    int bounce;
    int medium;  // extension dielectrics: bit 0 while the path is inside one, bit 1 once it carries l.x alone
    // Between a primary hit and its shadow ray:
    float3 nrm, shDir;
    float4 brdf;
    float brdfPdf, lightPdf, cosL, shLightID;
    int shObj;
    uint32_t ev;  // trace event word of the current bounce
};

// GenerateSeed + SSAA + camera + aperture + hero wavelength + TracePathLens +
// SampleWavelengths (SC:948-974, SC:1446-1472) for sample k of pixel
// (xx, yy) with uv the pixel's centre coordinate.
PT_DI void start_sample(PathState& ps, const KScene& S, const pt_push& pc, const CamInfo& cam, uint32_t xx,
                        uint32_t yy, float uvx, float uvy, int k) {
    const int W = pc.resolution[0], H = pc.resolution[1];
    uint32_t seed = pcg32((uint32_t)(pc.frame - pc.samplesPerFrame + k)) + (xx + (uint32_t)W * yy);
    const float jx = 2.0f * rnd(seed) - 0.5f;
    const float jy = 2.0f * rnd(seed) - 0.5f;
    const float sc = -pc.cameraSize * 0.5f;
    const float u = (uvx + jx / (float)W) * sc;
    const float v = (uvy + jy / (float)H) * sc;
    const float3 camPos = f3(pc.cameraPosX, pc.cameraPosY, pc.cameraPosZ);
    float3 org = camPos + mul_vm(f3(u, v, 0.0f), cam.cam);
    const float rx = rnd(seed);
    const float ry = rnd(seed);
    const float phi = 2.0f * PT_PI * ry;
    const float dd = sqrtf(rx);
    const float ha = 0.5f * pc.apertureSize;
    float sp, cp;
    ptm_sincosf(phi, &sp, &cp);
    const float3 poa = camPos + mul_vm(f3(ha * (dd * cp), ha * (dd * sp), pc.apertureDist), cam.cam);
    float3 dir = normalize3(poa - org);
    const bool xrange = (S.ext.flags & PT_EXT_WAVELENGTHS) != 0;
    const float lh = xrange ? mix_glsl(S.ext.lambda_min, S.ext.lambda_max, rnd(seed)) : mix_glsl(360.0f, 800.0f, rnd(seed));
    {
        LensGeom cl;
        cl.pos = cam.lensPos;
        cl.rot = cam.lensRot;
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
    if (xrange) {  // the hero and three rotations a quarter of the range apart
        const float lo = S.ext.lambda_min, R = S.ext.lambda_max - S.ext.lambda_min;
        const float base = lh - lo, q = R * 0.25f;
        ps.l = f4(lo + mod_glsl(base + q, R), lo + mod_glsl(base + q * 2.0f, R), lo + mod_glsl(base + q * 3.0f, R),
                  lo + mod_glsl(base + R, R));
    } else {
        const float base = lh - 390.0f;
        ps.l = f4(390.0f + mod_glsl(base + 82.5f, 330.0f), 390.0f + mod_glsl(base + 165.0f, 330.0f),
                  390.0f + mod_glsl(base + 247.5f, 330.0f), 390.0f + mod_glsl(base + 330.0f, 330.0f));
    }
    ps.org = org;
    ps.dir = dir;
    ps.seed = seed;
    ps.radiance = f4s(0.0f);
    ps.rr = f4s(1.0f);
    ps.mis = 1.0f;
    ps.bounce = 0;
    ps.medium = 0;
}

// What the caller does after a shading step.
enum StepResult {
    STEP_SHADOW = 0,       // trace ps.shDir from ps.org next
    STEP_CONTINUE = 1,     // bounce complete; trace ps.dir from ps.org next
    STEP_TERMINATED = 2,   // bounce complete; the path is finished
};

// BRDF throughput and Russian roulette, SC:1373-1385, then the pathLength
// check of TracePath (SC:1400).
template <bool TRACE>
PT_DI StepResult roulette(PathState& ps, int depth) {
    const float rp = fminf(fmaxf(fmaxf(ps.rr.x, fmaxf(ps.rr.y, fmaxf(ps.rr.z, ps.rr.w))), 0.0f), 0.99f);
    if (rnd(ps.seed) > rp) {
        if (TRACE) ps.ev |= PT_EV_RR_KILL;
        ps.bounce++;
        return STEP_TERMINATED;
    }
    ps.rr = ps.rr * (1.0f / rp);
    ps.bounce++;
    return (ps.bounce >= depth) ? STEP_TERMINATED : STEP_CONTINUE;
}
template <bool TRACE>
PT_DI StepResult finish_bounce(PathState& ps, int depth) {
    const float costheta = dot3(ps.dir, ps.nrm);
    ps.rr = ps.rr * ((ps.brdf * costheta) / ps.brdfPdf);
    return roulette<TRACE>(ps, depth);
}

// ---- extension surface models (PT_EXT_MATERIALS) ----
// The extension entry of a hit's material (0-based index floor(materialID)),
// or null for the reference's Lambertian.
PT_DI const pt_material_ext* ext_material(const KScene& S, float materialID) {
    if (!(S.ext.flags & PT_EXT_MATERIALS)) return nullptr;
    const int mi = (int)floorf(materialID);
    if (mi < 0 || mi >= S.ext.nmat || mi >= PT_MAX_EXT_MATERIALS) return nullptr;
    const pt_material_ext* m = &S.ext.mat[mi];
    return (m->type == PT_BSDF_REFERENCE) ? nullptr : m;
}
// Refractive index of an extension dielectric at wavelength l (nm).
PT_DI float ext_ior(const pt_material_ext& m, float l) {
    const float u = l * 1e-3f;
    const float u2 = u * u;
    if (m.type == PT_BSDF_CAUCHY) return m.p[0] + m.p[1] / u2;
    float n2 = 1.0f;
    n2 += (m.p[0] * u2) / (u2 - m.p[3]);
    n2 += (m.p[1] * u2) / (u2 - m.p[4]);
    n2 += (m.p[2] * u2) / (u2 - m.p[5]);
    return sqrtf(n2);
}
// Unpolarised Fresnel reflectance for relative index eta = n1 / n2 at
// incidence cosine cosi (>= 0); 1 under total internal reflection.  *cost
// receives the transmitted cosine.
PT_DI float fresnel_dielectric(float eta, float cosi, float* cost) {
    const float sin2t = (eta * eta) * (1.0f - cosi * cosi);
    if (sin2t >= 1.0f) {
        *cost = 0.0f;
        return 1.0f;
    }
    const float ct = sqrtf(1.0f - sin2t);
    const float rs = (eta * cosi - ct) / (eta * cosi + ct);
    const float rp = (cosi - eta * ct) / (cosi + eta * ct);
    *cost = ct;
    return 0.5f * (rs * rs + rp * rp);
}
// The reflectance of a Lambertian extension material at the four wavelengths, / PI.
PT_DI float4 ext_lambert(const pt_material_ext& m, float4 l) {
    if (m.type == PT_BSDF_FLAT) return f4s(m.p[0]) / PT_PI;
    const float4 x = f4((l.x - m.p[2]) / m.p[3], (l.y - m.p[2]) / m.p[3], (l.z - m.p[2]) / m.p[3],
                        (l.w - m.p[2]) / m.p[3]);
    const float4 v = f4(m.p[0] + m.p[1] * ptm_expf(-(x.x * x.x)), m.p[0] + m.p[1] * ptm_expf(-(x.y * x.y)),
                        m.p[0] + m.p[1] * ptm_expf(-(x.z * x.z)), m.p[0] + m.p[1] * ptm_expf(-(x.w * x.w)));
    return v / PT_PI;
}
// A specular bounce off a mirror or dielectric: the new direction from the
// hit point, the throughput, MIS weight 1 for the emitter the next ray may
// hit (no light sample was taken here), then Russian roulette.  Dielectrics
// choose reflection or transmission by the Fresnel reflectance at the first
// wavelength (l.x); a reflection keeps every wavelength, weighted by its own
// reflectance over the chosen one; a transmission bends each wavelength
// differently, so from the first transmission on the path carries l.x
// alone, with 4x its throughput (the sample's colour averages the four
// wavelengths).  Returns the step result.
template <bool TRACE>
PT_DI StepResult shade_specular(PathState& ps, const pt_material_ext& m, const Hit& h, int depth) {
    ps.org = fma3s(ps.dir, h.hitdist, ps.org);
    float3 n = h.normal;
    float c = dot3(ps.dir, n);
    if (c > 0.0f) {  // face the incoming ray
        n = f3(-n.x, -n.y, -n.z);
        c = -c;
    }
    ps.nrm = n;
    ps.mis = 1.0f;
    const float cosi = -c;
    if (m.type == PT_BSDF_MIRROR) {
        ps.dir = ps.dir + n * (2.0f * cosi);
        ps.rr = ps.rr * m.p[0];
        if (TRACE) ps.ev |= PT_EV_SPECULAR;
        return roulette<TRACE>(ps, depth);
    }
    const bool inside = (ps.medium & 1) != 0;
    const float nh = ext_ior(m, ps.l.x);
    const float eta = inside ? nh : 1.0f / nh;
    float cost = 0.0f;
    const float F = fresnel_dielectric(eta, cosi, &cost);
    if (rnd(ps.seed) < F) {
        ps.dir = ps.dir + n * (2.0f * cosi);
        float ct;
        const float ny = ext_ior(m, ps.l.y), nz = ext_ior(m, ps.l.z), nw = ext_ior(m, ps.l.w);
        const float Fy = fresnel_dielectric(inside ? ny : 1.0f / ny, cosi, &ct);
        const float Fz = fresnel_dielectric(inside ? nz : 1.0f / nz, cosi, &ct);
        const float Fw = fresnel_dielectric(inside ? nw : 1.0f / nw, cosi, &ct);
        ps.rr = f4(ps.rr.x, ps.rr.y * (Fy / F), ps.rr.z * (Fz / F), ps.rr.w * (Fw / F));
        if (TRACE) ps.ev |= PT_EV_SPECULAR;
    } else {
        ps.dir = normalize3(ps.dir * eta + n * (eta * cosi - cost));
        if (!(ps.medium & 2)) {  // the first transmission: l.x alone from here on
            ps.rr = f4(ps.rr.x * 4.0f, 0.0f, 0.0f, 0.0f);
            ps.medium |= 2;
        }
        ps.medium ^= 1;
        if (TRACE) ps.ev |= PT_EV_REFRACT;
    }
    return roulette<TRACE>(ps, depth);
}

// TraceRay after Intersection (SC:1345-1391) for the path ray: emitter, miss,
// or BRDF sampling + SampleLightSource (SC:1298-1343) up to the shadow ray.
template <bool TRACE>
PT_DI StepResult shade_primary(PathState& ps, const KScene& S, const Hit& h, int objectID, int depth) {
    if (TRACE) ps.ev = PT_EV_VALID;
    if (!(h.hitdist < PT_MAXDIST)) {
        if (TRACE) ps.ev |= PT_EV_HIT_MISS;
        if (S.ext.flags & PT_EXT_SKY) {  // no light sample reaches the sky: weight 1
            ps.radiance = ps.radiance + emit(ps.l, S.ext.sky_temperature, S.ext.sky_luminosity) * ps.rr;
        } else {
            ps.radiance = ps.radiance + f4s(0.0f);
        }
        ps.bounce++;
        return STEP_TERMINATED;
    }
    if (TRACE) ps.ev |= (objectID == -2) ? PT_EV_HIT_SDF : ((uint32_t)objectID & PT_EV_HIT_MASK);
    const float2 lt = light_mix(S, h.lightID);
    if (lt.y > 0.0f) {
        ps.radiance = ps.radiance + (emit(ps.l, lt.x, lt.y) * ps.rr) * ps.mis;
        if (TRACE) ps.ev |= PT_EV_EMITTER;
        ps.bounce++;
        return STEP_TERMINATED;
    }
    const pt_material_ext* xm = ext_material(S, h.materialID);
    if (xm && xm->type >= PT_BSDF_MIRROR) return shade_specular<TRACE>(ps, *xm, h, depth);
    if (xm) {
        ps.brdf = ext_lambert(*xm, ps.l);
    } else {
        const float3 mat = material_mix(S, h.materialID);
        ps.brdf = evaluate_brdf(ps.l, mat.x, mat.y, mat.z);
    }
    ps.nrm = h.normal;
    ps.org = fma3s(ps.dir, h.hitdist, ps.org);
    {  // SampleBRDF: cosine direction via the unit sphere, SC:984-1003.
        const float rx = rnd(ps.seed);
        const float ry = rnd(ps.seed);
        const float phi = 2.0f * PT_PI * ry;
        const float sinTheta = 2.0f * rx - 1.0f;
        const float cosTheta = sqrtf(__fmaf_rn(-sinTheta, sinTheta, 1.0f));
        float sp, cp;
        ptm_sincosf(phi, &sp, &cp);
        ps.dir = normalize3(ps.nrm + f3(cp * cosTheta, sp * cosTheta, sinTheta));
    }
    ps.brdfPdf = dot3(ps.dir, ps.nrm) / PT_PI;
    const float numLights = S.numObjects[6];
    int pick = 0;
    uint32_t shadowState = 0;
    bool shadow = false;
    if (numLights > 0.0f) {
        float boundingRadius = 0.0f;
        float3 lightPos = f3(0.0f, 0.0f, 0.0f);
        ps.shLightID = -1.0f;
        ps.shObj = sample_random_light(S, ps.seed, boundingRadius, lightPos, ps.shLightID, pick);
        const float invLightDistance = 1.0f / length3(lightPos - ps.org);
        const float3 lightDir = (lightPos - ps.org) * invLightDistance;
        const float sinthetaMax = fminf(boundingRadius * invLightDistance, 1.0f);
        const float costhetaMax = sqrtf(1.0f - sinthetaMax * sinthetaMax);
        {  // SampleCosineUnitCone, SC:1012-1023.
            const float rx = rnd(ps.seed);
            const float ry = rnd(ps.seed);
            const float cosAlphaMax = 2.0f * costhetaMax * costhetaMax - 1.0f;
            const float phi = 2.0f * PT_PI * ry;
            const float cosTheta = (1.0f - cosAlphaMax) * rx + cosAlphaMax;
            const float sinTheta = sqrtf(__fmaf_rn(-cosTheta, cosTheta, 1.0f));
            float sp, cp;
            ptm_sincosf(phi, &sp, &cp);
            ps.shDir = to_world(normalize3(f3(cp * sinTheta, sp * sinTheta, cosTheta + 1.0f)), lightDir);
        }
        ps.lightPdf = 1.0f / numLights;
        ps.lightPdf *= dot3(ps.shDir, lightDir) / (PT_PI * (1.0f - costhetaMax * costhetaMax));
        ps.mis = ps.brdfPdf * ps.brdfPdf / (ps.brdfPdf * ps.brdfPdf + ps.lightPdf * ps.lightPdf);
        ps.cosL = dot3(ps.shDir, ps.nrm);
        const float deathProbability = 1.25f * fmaxf(ps.mis - 0.2f, 0.0f);
        if (ps.cosL >= 0.0f) {
            if (rnd(ps.seed) > deathProbability) {
                shadow = true;
            } else {
                ps.mis = 1.0f;
                shadowState = 1;
            }
        }
    } else {
        ps.mis = ps.brdfPdf * ps.brdfPdf / (ps.brdfPdf * ps.brdfPdf + 0.0f * 0.0f);
    }
    if (TRACE) ps.ev |= ((uint32_t)(pick & 0x7F) << PT_EV_LIGHT_SHIFT) | (shadowState << PT_EV_SHADOW_SHIFT);
    if (shadow) return STEP_SHADOW;
    ps.radiance = ps.radiance + f4s(0.0f);
    return finish_bounce<TRACE>(ps, depth);
}

// LightSourceVisibilityCheck result (SC:1121-1223) and the NEE term, then the
// rest of the bounce.
template <bool TRACE>
PT_DI StepResult shade_shadow(PathState& ps, const KScene& S, int objectID, int depth) {
    const int obj = (objectID == -2) ? -1 : objectID;
    float4 contrib = f4s(0.0f);
    if (obj == ps.shObj) {
        const float2 lt = light_mix(S, ps.shLightID);
        const float4 rrl = ps.rr * ((ps.brdf * ps.cosL) / ps.lightPdf);
        contrib = (emit(ps.l, lt.x, lt.y) * rrl) * (1.0f - ps.mis);
        if (TRACE) ps.ev |= 3u << PT_EV_SHADOW_SHIFT;
    } else {
        if (TRACE) ps.ev |= 2u << PT_EV_SHADOW_SHIFT;
    }
    ps.radiance = ps.radiance + contrib;
    return finish_bounce<TRACE>(ps, depth);
}

// SC:1477-1489: the sample's XYZ with NaN rejection.
PT_DI float3 sample_color(const PathState& ps, const KScene& S, const float* __restrict__ cie) {
    float3 wx, wy, wz, ww;
    if (S.ext.flags & PT_EXT_ANALYTIC_CMF) {
        wx = cmf_analytic(ps.l.x);
        wy = cmf_analytic(ps.l.y);
        wz = cmf_analytic(ps.l.z);
        ww = cmf_analytic(ps.l.w);
    } else {
        wx = wave_to_xyz(cie, ps.l.x);
        wy = wave_to_xyz(cie, ps.l.y);
        wz = wave_to_xyz(cie, ps.l.z);
        ww = wave_to_xyz(cie, ps.l.w);
    }
    // 1 / pdf of a wavelength: the width of the range it is uniform over
    const float range = (S.ext.flags & PT_EXT_WAVELENGTHS) ? (S.ext.lambda_max - S.ext.lambda_min) : (720.0f - 390.0f);
    float3 color = (((wx * ps.radiance.x + wy * ps.radiance.y) + wz * ps.radiance.z) + ww * ps.radiance.w) * range *
                   0.25f;
    if (color.x != color.x || color.y != color.y || color.z != color.z) color = f3(0.0f, 0.0f, 0.0f);
    return color;
}

// Rendering + Accumulate, SC:1513-1520, SC:1492-1507: the pixel's new value
// from the ordered sample sum and the old accumulator value.
PT_DI float4 accumulate(const pt_push& pc, float3 sum, float4 old) {
    const float fs = (float)pc.samplesPerFrame;
    float3 out = f3(sum.x / fs, sum.y / fs, sum.z / fs);
    out = out * (pc.apertureSize * pc.apertureSize * (float)pc.ISO);
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
    return make_float4(out.x, out.y, out.z, 1.0f);
}
