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
// float(seed) / float(0xFFFFFFFFu): round-to-nearest conversion, divisor
// 2^32 (the double renderer converts exactly and can never reach 1.0).
template <typename R = float> PT_DI R rnd(uint32_t& seed);
template <> PT_DI float rnd<float>(uint32_t& seed) {
    seed = pcg32(seed);
    return __uint2float_rn(seed) / 4294967296.0f;
}
template <> PT_DI double rnd<double>(uint32_t& seed) {
    seed = pcg32(seed);
    return (double)seed / 4294967296.0;
}

// WaveToXYZ, SC:129-140, from the CIE table in global memory.
PT_DI float cie_at(const float* __restrict__ cie, int i) {
    return ((unsigned)i < (unsigned)PT_CIE_TABLE_SIZE) ? __ldg(cie + i) : 0.0f;
}
// One lobe of the multi-lobe Gaussian CIE fit (Wyman, Sloan and Shirley
// 2013): a Gaussian with a different width on each side of its peak.
template <typename R> PT_DI R cmf_lobe(R x, R mu, R s1, R s2) {
    const R t = (x - mu) / ((x < mu) ? s1 : s2);
    return m_exp(-PT_LIT(R, 0.5) * t * t);
}
// The fit itself at wavelength `wave` (nm), for PT_EXT_ANALYTIC_CMF.
template <typename R> PT_DI V3<R> cmf_analytic(R wave) {
    const R x = (PT_LIT(R, 1.056) * cmf_lobe(wave, PT_LIT(R, 599.8), PT_LIT(R, 37.9), PT_LIT(R, 31.0)) + PT_LIT(R, 0.362) * cmf_lobe(wave, PT_LIT(R, 442.0), PT_LIT(R, 16.0), PT_LIT(R, 26.7))) -
                    PT_LIT(R, 0.065) * cmf_lobe(wave, PT_LIT(R, 501.1), PT_LIT(R, 20.4), PT_LIT(R, 26.2));
    const R y = PT_LIT(R, 0.821) * cmf_lobe(wave, PT_LIT(R, 568.8), PT_LIT(R, 46.9), PT_LIT(R, 40.5)) + PT_LIT(R, 0.286) * cmf_lobe(wave, PT_LIT(R, 530.9), PT_LIT(R, 16.3), PT_LIT(R, 31.1));
    const R z = PT_LIT(R, 1.217) * cmf_lobe(wave, PT_LIT(R, 437.0), PT_LIT(R, 11.8), PT_LIT(R, 36.0)) + PT_LIT(R, 0.681) * cmf_lobe(wave, PT_LIT(R, 459.0), PT_LIT(R, 26.0), PT_LIT(R, 13.8));
    return v3<R>(x, y, z);
}
template <typename R> PT_DI V3<R> wave_to_xyz(const float* __restrict__ cie, R wave) {
    V3<R> r = v3<R>(PT_LIT(R, 0.0), PT_LIT(R, 0.0), PT_LIT(R, 0.0));
    if ((wave >= PT_LIT(R, 360.0)) && (wave <= PT_LIT(R, 800.0))) {
        const int i3 = 3 * (int)(m_floor(wave) - PT_LIT(R, 360.0));
        const R a = wave - m_floor(wave);
        r = v3<R>(mix_glsl<R>(cie_at(cie, i3), cie_at(cie, i3 + 3), a),
                  mix_glsl<R>(cie_at(cie, i3 + 1), cie_at(cie, i3 + 4), a),
                  mix_glsl<R>(cie_at(cie, i3 + 2), cie_at(cie, i3 + 5), a));
    }
    return r;
}

// SpectralPowerDistribution / EvaluateBRDF, SC:1030-1038, SC:1075-1080.
template <typename V, typename R = SOf<V>> PT_DI V evaluate_brdf(V l, ND<R> peak, ND<R> sigma, ND<R> invertf) {
    const R den = PT_LIT(R, 2.0) * sigma * sigma;
    const V4<R> x = v4<R>((l.x - peak) / den, (l.y - peak) / den, (l.z - peak) / den, (l.w - peak) / den);
    const V4<R> r = v4<R>(m_exp(-x.x * x.x), m_exp(-x.y * x.y), m_exp(-x.z * x.z), m_exp(-x.w * x.w));
    const R a = (R)(int)invertf;
    const V4<R> s = v4<R>(mix_glsl(r.x, PT_LIT(R, 1.0) - r.x, a), mix_glsl(r.y, PT_LIT(R, 1.0) - r.y, a), mix_glsl(r.z, PT_LIT(R, 1.0) - r.z, a),
                        mix_glsl(r.w, PT_LIT(R, 1.0) - r.w, a));
    return s / PT_PI_R(R);
}

// BlackBodyRadiation / Emit, SC:1040-1055.
// pow(l, -5) as ptm_powf computes it, 1 / l^5 by binary powering (l > 0).
template <typename R> PT_DI R blackbody(R l, R T) {
    return (PT_LIT(R, 1.1910429724e-16) * (PT_LIT(R, 1.0) / pow_pos_int<5>(l))) / (m_exp(PT_LIT(R, 0.014387768775) / (l * T)) - PT_LIT(R, 1.0));
}
template <typename V, typename R = SOf<V>> PT_DI V emit(V l, ND<R> temperature_in, ND<R> luminosity) {
    const R T = m_fmax(temperature_in, PT_LIT(R, 0.0));
    const V4<R> lm = l * PT_LIT(R, 1e-9);
    const R peak = PT_LIT(R, 4.0956746759e-6) * pow_pos_int<5>(T);  // T >= 0
    const V4<R> e = v4<R>(blackbody(lm.x, T) / peak, blackbody(lm.y, T) / peak, blackbody(lm.z, T) / peak,
                        blackbody(lm.w, T) / peak);
    return e * m_fmax(luminosity, PT_LIT(R, 0.0));
}

// RefractiveIndexBK7Glass, SC:1064-1073.
template <typename R> PT_DI R bk7_index(R l) {
    l *= PT_LIT(R, 1e-3);
    const R l2 = l * l;
    R n2 = PT_LIT(R, 1.0);
    n2 += (PT_LIT(R, 1.03961212) * l2) / (l2 - PT_LIT(R, 6.00069867e-3));
    n2 += (PT_LIT(R, 0.231792344) * l2) / (l2 - PT_LIT(R, 2.00179144e-2));
    n2 += (PT_LIT(R, 1.01046945) * l2) / (l2 - PT_LIT(R, 1.03560653e2));
    return m_sqrt(n2);
}

// OrthonormalBasis + ToWorld, SC:1093-1119.
template <typename V, typename R = SOf<V>> PT_DI V to_world(V v, V n) {
    V3<R> b1 = v3<R>(PT_LIT(R, 0.0), -PT_LIT(R, 1.0), PT_LIT(R, 0.0));
    V3<R> b2 = v3<R>(-PT_LIT(R, 1.0), PT_LIT(R, 0.0), PT_LIT(R, 0.0));
    if (n.z >= -PT_LIT(R, 0.9999999)) {
        const R a = PT_LIT(R, 1.0) / (PT_LIT(R, 1.0) + n.z);
        const R b = -n.x * n.y * a;
        b1 = v3<R>(PT_LIT(R, 1.0) - (n.x * n.x * a), b, -n.x);
        b2 = v3<R>(b, PT_LIT(R, 1.0) - (n.y * n.y * a), -n.y);
    }
    return b1 * v.x + b2 * v.y + n * v.z;
}

// GetMaterialMix, SC:237-249.
template <typename R> PT_DI V3<R> material_mix(const KScene& S, R materialID) {
    const int i1 = 3 * (int)m_floor(materialID);
    const int i2 = 3 * (int)m_ceil(materialID);
    const R x = materialID - m_floor(materialID);
    return v3<R>(mix_glsl<R>(s_mat(S, i1), s_mat(S, i2), x), mix_glsl<R>(s_mat(S, i1 + 1), s_mat(S, i2 + 1), x),
                 mix_glsl<R>(s_mat(S, i1 + 2), s_mat(S, i2 + 2), x));
}
// UnpackLight via GetLightMix, SC:224-235, SC:251-254.
template <typename R> PT_DI V2<R> light_mix(const KScene& S, R lightID) {
    const int index = (int)lightID;
    if (index == -1) return v2<R>(PT_LIT(R, 5500.0), PT_LIT(R, 0.0));
    return v2<R>(s_light(S, 2 * index), s_light(S, 2 * index + 1));
}

// SampleRandomLightSource, SC:1225-1285, quirks included: the lens branch
// compares with the box count (SC:1264) and the cyclide branch with the lens
// count (SC:1275).  Object reads are guarded: these indices come from data.
template <typename R>
PT_DI int sample_random_light(const KScene& S, uint32_t& seed, R& boundingRadius, V3<R>& pos, R& lightID,
                              int& pick) {
    const int randomLight = (int)m_floor(rnd<R>(seed) * S.numObjects[6]);
    pick = randomLight;
    const int result = (int)s_lightid(S, randomLight);
    int L = result;
    int offset = 0;
    const int* n = S.meta.n;
    if (L < n[0]) {
        const int b = 6 * L;
        boundingRadius = s_obj(S, b + 3);
        pos = v3<R>(s_obj(S, b), s_obj(S, b + 1), s_obj(S, b + 2));
        lightID = (R)((int)s_obj(S, b + 5) - 1);
        return result;
    }
    L -= n[0];
    offset += 6 * n[0];
    if (L < n[1]) {
        const int b = 5 * L + offset;
        boundingRadius = PT_LIT(R, 1e5);
        pos = v3<R>(s_obj(S, b), s_obj(S, b + 1), s_obj(S, b + 2));
        lightID = (R)((int)s_obj(S, b + 4) - 1);
        return result;
    }
    L -= n[1];
    offset += 5 * n[1];
    if (L < n[2]) {
        const int b = 11 * L + offset;
        boundingRadius = PT_LIT(R, 0.5) * length3(v3<R>(s_obj(S, b + 6), s_obj(S, b + 7), s_obj(S, b + 8)));
        pos = v3<R>(s_obj(S, b), s_obj(S, b + 1), s_obj(S, b + 2));
        lightID = (R)((int)s_obj(S, b + 10) - 1);
        return result;
    }
    L -= n[2];
    offset += 11 * n[2];
    if (L < n[2]) {
        const int b = 12 * L + offset;
        const R r = s_obj(S, b + 6), th = s_obj(S, b + 8);
        boundingRadius = m_sqrt((r * r) + (PT_LIT(R, 0.25) * th * th));
        pos = v3<R>(s_obj(S, b), s_obj(S, b + 1), s_obj(S, b + 2));
        lightID = (R)((int)s_obj(S, b + 11) - 1);
        return result;
    }
    L -= n[3];
    offset += 12 * n[3];
    if (L < n[3]) {
        const int b = 16 * L + offset;
        boundingRadius = m_sqrt(s_obj(S, b + 13));
        pos = v3<R>(s_obj(S, b), s_obj(S, b + 1), s_obj(S, b + 2));
        lightID = (R)((int)s_obj(S, b + 15) - 1);
        return result;
    }
    return 0;
}


template <typename R = float> PT_DI CamInfoT<R> make_camera(const pt_push& pc) {
    CamInfoT<R> c;
    c.cam = rotation_matrix(v3<R>(pc.cameraAngle[0], pc.cameraAngle[1], PT_LIT(R, 0.0)));
    const V3<R> camPos = v3<R>(pc.cameraPosX, pc.cameraPosY, pc.cameraPosZ);
    const V3<R> fwd = v3<R>(c.cam.c0.z, c.cam.c1.z, c.cam.c2.z);
    c.lensRot = rotation_matrix(v3<R>(PT_LIT(R, 0.0), PT_LIT(R, 90.0) - pc.cameraAngle[1], pc.cameraAngle[0]));
    c.lensPos = camPos + fwd * pc.lensDistance;
    return c;
}

// The state of one camera path between scene intersections.
template <typename R> struct PathStateT {
    V3<R> org, dir;         // path ray (after a non-emissive hit: the new origin and the BRDF direction)
    V4<R> l, radiance, rr;  // wavelengths, accumulated radiance, throughput
    R mis;               // MISBRDFWeight
    uint32_t seed;
    int bounce;
    int medium;  // extension dielectrics: bit 0 while the path is inside one, bit 1 once it carries l.x alone
    // Between a primary hit and its shadow ray:
    V3<R> nrm, shDir;
    V4<R> brdf;
    R brdfPdf, lightPdf, cosL, shLightID;
    int shObj;
    uint32_t ev;  // trace event word of the current bounce
};
using PathState = PathStateT<float>;

// GenerateSeed + SSAA + camera + aperture + hero wavelength + TracePathLens +
// SampleWavelengths (SC:948-974, SC:1446-1472) for sample k of pixel
// (xx, yy) with uv the pixel's centre coordinate.
template <typename R>
PT_DI void start_sample(PathStateT<R>& ps, const KScene& S, const pt_push& pc, const CamInfoT<R>& cam, uint32_t xx,
                        uint32_t yy, ND<R> uvx, ND<R> uvy, int k) {
    const int W = pc.resolution[0], H = pc.resolution[1];
    uint32_t seed = pcg32((uint32_t)(pc.frame - pc.samplesPerFrame + k)) + (xx + (uint32_t)W * yy);
    const R jx = PT_LIT(R, 2.0) * rnd<R>(seed) - PT_LIT(R, 0.5);
    const R jy = PT_LIT(R, 2.0) * rnd<R>(seed) - PT_LIT(R, 0.5);
    const R sc = -pc.cameraSize * PT_LIT(R, 0.5);
    const R u = (uvx + jx / (R)W) * sc;
    const R v = (uvy + jy / (R)H) * sc;
    const V3<R> camPos = v3<R>(pc.cameraPosX, pc.cameraPosY, pc.cameraPosZ);
    V3<R> org = camPos + mul_vm(v3<R>(u, v, PT_LIT(R, 0.0)), cam.cam);
    const R rx = rnd<R>(seed);
    const R ry = rnd<R>(seed);
    const R phi = PT_LIT(R, 2.0) * PT_PI_R(R) * ry;
    const R dd = m_sqrt(rx);
    const R ha = PT_LIT(R, 0.5) * pc.apertureSize;
    R sp, cp;
    m_sincos(phi, &sp, &cp);
    const V3<R> poa = camPos + mul_vm(v3<R>(ha * (dd * cp), ha * (dd * sp), pc.apertureDist), cam.cam);
    V3<R> dir = normalize3(poa - org);
    const bool xrange = (S.ext.flags & PT_EXT_WAVELENGTHS) != 0;
    const R lh = xrange ? mix_glsl<R>(S.ext.lambda_min, S.ext.lambda_max, rnd<R>(seed))
                        : mix_glsl(PT_LIT(R, 360.0), PT_LIT(R, 800.0), rnd<R>(seed));
    {
        LensGeomT<R> cl;
        cl.pos = cam.lensPos;
        cl.rot = cam.lensRot;
        cl.radius = pc.lensRadius;
        cl.focal = pc.lensFocalLength;
        cl.thickness = pc.lensThickness;
        cl.converging = true;
        R lam = lh;
#pragma unroll 1
        for (int i = 0; i < 2; i++) {
            HitT<R> h;
            h.hitdist = PT_LIT(R, 1e6);
            h.normal = v3<R>(PT_LIT(R, 0.0), PT_LIT(R, 0.0), PT_LIT(R, 0.0));
            h.materialID = PT_LIT(R, 0.0);
            h.lightID = -PT_LIT(R, 1.0);
            int isOutside = 1;
            lens_intersect(org, dir, cl, PT_LIT(R, 0.0), -PT_LIT(R, 1.0), h, isOutside);
            R n1, n2;
            if (isOutside == 1) {
                n1 = PT_LIT(R, 1.0);
                n2 = bk7_index(lam);
            } else {
                n1 = bk7_index(lam);
                n2 = PT_LIT(R, 1.0);
            }
            const R n12 = n1 / n2;
            lam = lam * n12;
            org = fma3s(dir, h.hitdist, org);
            dir = refract3(dir, h.normal, n12);
        }
    }
    if (xrange) {  // the hero and three rotations a quarter of the range apart
        const R lo = S.ext.lambda_min, Rw = S.ext.lambda_max - S.ext.lambda_min;
        const R base = lh - lo, q = Rw * PT_LIT(R, 0.25);
        ps.l = v4<R>(lo + mod_glsl(base + q, Rw), lo + mod_glsl(base + q * PT_LIT(R, 2.0), Rw),
                     lo + mod_glsl(base + q * PT_LIT(R, 3.0), Rw), lo + mod_glsl(base + Rw, Rw));
    } else {
        const R base = lh - PT_LIT(R, 390.0);
        ps.l = v4<R>(PT_LIT(R, 390.0) + mod_glsl(base + PT_LIT(R, 82.5), PT_LIT(R, 330.0)), PT_LIT(R, 390.0) + mod_glsl(base + PT_LIT(R, 165.0), PT_LIT(R, 330.0)),
                  PT_LIT(R, 390.0) + mod_glsl(base + PT_LIT(R, 247.5), PT_LIT(R, 330.0)), PT_LIT(R, 390.0) + mod_glsl(base + PT_LIT(R, 330.0), PT_LIT(R, 330.0)));
    }
    ps.org = org;
    ps.dir = dir;
    ps.seed = seed;
    ps.radiance = v4s<R>(PT_LIT(R, 0.0));
    ps.rr = v4s<R>(PT_LIT(R, 1.0));
    ps.mis = PT_LIT(R, 1.0);
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
template <bool TRACE, typename R>
PT_DI StepResult roulette(PathStateT<R>& ps, int depth) {
    const R rp = m_fmin(m_fmax(m_fmax(ps.rr.x, m_fmax(ps.rr.y, m_fmax(ps.rr.z, ps.rr.w))), PT_LIT(R, 0.0)), PT_LIT(R, 0.99));
    if (rnd<R>(ps.seed) > rp) {
        if (TRACE) ps.ev |= PT_EV_RR_KILL;
        ps.bounce++;
        return STEP_TERMINATED;
    }
    ps.rr = ps.rr * (PT_LIT(R, 1.0) / rp);
    ps.bounce++;
    return (ps.bounce >= depth) ? STEP_TERMINATED : STEP_CONTINUE;
}
// The bounce's throughput update (SC:1373-1374, before the roulette).
template <typename R> PT_DI V4<R> bounce_throughput(const PathStateT<R>& ps) {
    const R costheta = dot3(ps.dir, ps.nrm);
    return ps.rr * ((ps.brdf * costheta) / ps.brdfPdf);
}
template <bool TRACE, typename R>
PT_DI StepResult finish_bounce(PathStateT<R>& ps, int depth) {
    ps.rr = bounce_throughput(ps);
    return roulette<TRACE>(ps, depth);
}

// ---- extension surface models (PT_EXT_MATERIALS) ----
// The extension entry of a hit's material (0-based index floor(materialID)),
// or null for the reference's Lambertian.
template <typename R> PT_DI const pt_material_ext* ext_material(const KScene& S, R materialID) {
    if (!(S.ext.flags & PT_EXT_MATERIALS)) return nullptr;
    const int mi = (int)m_floor(materialID);
    if (mi < 0 || mi >= S.ext.nmat || mi >= PT_MAX_EXT_MATERIALS) return nullptr;
    const pt_material_ext* m = &S.ext.mat[mi];
    return (m->type == PT_BSDF_REFERENCE) ? nullptr : m;
}
// Refractive index of an extension dielectric at wavelength l (nm).
template <typename R> PT_DI R ext_ior(const pt_material_ext& m, R l) {
    const R u = l * PT_LIT(R, 1e-3);
    const R u2 = u * u;
    if (m.type == PT_BSDF_CAUCHY) return m.p[0] + m.p[1] / u2;
    R n2 = PT_LIT(R, 1.0);
    n2 += (m.p[0] * u2) / (u2 - m.p[3]);
    n2 += (m.p[1] * u2) / (u2 - m.p[4]);
    n2 += (m.p[2] * u2) / (u2 - m.p[5]);
    return m_sqrt(n2);
}
// Unpolarised Fresnel reflectance for relative index eta = n1 / n2 at
// incidence cosine cosi (>= 0); 1 under total internal reflection.  *cost
// receives the transmitted cosine.
template <typename R> PT_DI R fresnel_dielectric(R eta, R cosi, R* cost) {
    const R sin2t = (eta * eta) * (PT_LIT(R, 1.0) - cosi * cosi);
    if (sin2t >= PT_LIT(R, 1.0)) {
        *cost = PT_LIT(R, 0.0);
        return PT_LIT(R, 1.0);
    }
    const R ct = m_sqrt(PT_LIT(R, 1.0) - sin2t);
    const R rs = (eta * cosi - ct) / (eta * cosi + ct);
    const R rp = (cosi - eta * ct) / (cosi + eta * ct);
    *cost = ct;
    return PT_LIT(R, 0.5) * (rs * rs + rp * rp);
}
// The reflectance of a Lambertian extension material at the four wavelengths, / PI.
template <typename V, typename R = SOf<V>> PT_DI V ext_lambert(const pt_material_ext& m, V l) {
    if (m.type == PT_BSDF_FLAT) return v4s<R>(m.p[0]) / PT_PI_R(R);
    const V4<R> x = v4<R>((l.x - m.p[2]) / m.p[3], (l.y - m.p[2]) / m.p[3], (l.z - m.p[2]) / m.p[3],
                        (l.w - m.p[2]) / m.p[3]);
    const V4<R> v = v4<R>(m.p[0] + m.p[1] * m_exp(-(x.x * x.x)), m.p[0] + m.p[1] * m_exp(-(x.y * x.y)),
                        m.p[0] + m.p[1] * m_exp(-(x.z * x.z)), m.p[0] + m.p[1] * m_exp(-(x.w * x.w)));
    return v / PT_PI_R(R);
}
// A specular bounce off a mirror or dielectric: the new direction from the
// hit point, the throughput, MIS weight 1 for the emitter the next ray may
// hit (no light sample was taken here), then Russian roulette.  Dielectrics
// choose reflection or transmission by the Fresnel reflectance at the first
// wavelength (l.x); a reflection keeps every wavelength, weighted by its own
// reflectance over the chosen one; a transmission bends each wavelength
// differently, so from the first transmission on the path carries l.x
// alone, with 4x its throughput (the sample's colour averages the four
// wavelengths).  The new ray starts 2e-4 along its direction: from the
// surface point itself, the sphere test's near root can round to a tiny
// positive distance, below the 1e-4 hit threshold, and a ray entering a
// glass sphere would then miss its far side.  Returns the step result.
template <bool TRACE, typename R>
PT_DI StepResult shade_specular(PathStateT<R>& ps, const pt_material_ext& m, const HitT<R>& h, int depth) {
    ps.org = fma3s(ps.dir, h.hitdist, ps.org);
    V3<R> n = h.normal;
    R c = dot3(ps.dir, n);
    if (c > PT_LIT(R, 0.0)) {  // face the incoming ray
        n = v3<R>(-n.x, -n.y, -n.z);
        c = -c;
    }
    ps.nrm = n;
    ps.mis = PT_LIT(R, 1.0);
    const R cosi = -c;
    if (m.type == PT_BSDF_MIRROR) {
        ps.dir = ps.dir + n * (PT_LIT(R, 2.0) * cosi);
        ps.org = fma3s(ps.dir, PT_LIT(R, 2e-4), ps.org);
        ps.rr = ps.rr * m.p[0];
        if (TRACE) ps.ev |= PT_EV_SPECULAR;
        return roulette<TRACE>(ps, depth);
    }
    const bool inside = (ps.medium & 1) != 0;
    const R nh = ext_ior(m, ps.l.x);
    const R eta = inside ? nh : PT_LIT(R, 1.0) / nh;
    R cost = PT_LIT(R, 0.0);
    const R F = fresnel_dielectric(eta, cosi, &cost);
    if (rnd<R>(ps.seed) < F) {
        ps.dir = ps.dir + n * (PT_LIT(R, 2.0) * cosi);
        R ct;
        const R ny = ext_ior(m, ps.l.y), nz = ext_ior(m, ps.l.z), nw = ext_ior(m, ps.l.w);
        const R Fy = fresnel_dielectric(inside ? ny : PT_LIT(R, 1.0) / ny, cosi, &ct);
        const R Fz = fresnel_dielectric(inside ? nz : PT_LIT(R, 1.0) / nz, cosi, &ct);
        const R Fw = fresnel_dielectric(inside ? nw : PT_LIT(R, 1.0) / nw, cosi, &ct);
        ps.rr = v4<R>(ps.rr.x, ps.rr.y * (Fy / F), ps.rr.z * (Fz / F), ps.rr.w * (Fw / F));
        if (TRACE) ps.ev |= PT_EV_SPECULAR;
    } else {
        ps.dir = normalize3(ps.dir * eta + n * (eta * cosi - cost));
        if (!(ps.medium & 2)) {  // the first transmission: l.x alone from here on
            ps.rr = v4<R>(ps.rr.x * PT_LIT(R, 4.0), PT_LIT(R, 0.0), PT_LIT(R, 0.0), PT_LIT(R, 0.0));
            ps.medium |= 2;
        }
        ps.medium ^= 1;
        if (TRACE) ps.ev |= PT_EV_REFRACT;
    }
    ps.org = fma3s(ps.dir, PT_LIT(R, 2e-4), ps.org);
    return roulette<TRACE>(ps, depth);
}

// TraceRay after Intersection (SC:1345-1391) for the path ray: emitter, miss,
// or BRDF sampling + SampleLightSource (SC:1298-1343) up to the shadow ray.
template <bool TRACE, typename R>
PT_DI StepResult shade_primary(PathStateT<R>& ps, const KScene& S, const HitT<R>& h, int objectID, int depth) {
    if (TRACE) ps.ev = PT_EV_VALID;
    if (!(h.hitdist < R(PT_MAXDIST))) {
        if (TRACE) ps.ev |= PT_EV_HIT_MISS;
        if (S.ext.flags & PT_EXT_SKY) {  // no light sample reaches the sky: weight 1
            ps.radiance = ps.radiance + emit(ps.l, S.ext.sky_temperature, S.ext.sky_luminosity) * ps.rr;
        } else {
            ps.radiance = ps.radiance + v4s<R>(PT_LIT(R, 0.0));
        }
        ps.bounce++;
        return STEP_TERMINATED;
    }
    if (TRACE) ps.ev |= (objectID == -2) ? PT_EV_HIT_SDF : ((uint32_t)objectID & PT_EV_HIT_MASK);
    const V2<R> lt = light_mix(S, h.lightID);
    if (lt.y > PT_LIT(R, 0.0)) {
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
        const V3<R> mat = material_mix(S, h.materialID);
        ps.brdf = evaluate_brdf(ps.l, mat.x, mat.y, mat.z);
    }
    ps.nrm = h.normal;
    ps.org = fma3s(ps.dir, h.hitdist, ps.org);
    {  // SampleBRDF: cosine direction via the unit sphere, SC:984-1003.
        const R rx = rnd<R>(ps.seed);
        const R ry = rnd<R>(ps.seed);
        const R phi = PT_LIT(R, 2.0) * PT_PI_R(R) * ry;
        const R sinTheta = PT_LIT(R, 2.0) * rx - PT_LIT(R, 1.0);
        const R cosTheta = m_sqrt(m_fma(-sinTheta, sinTheta, PT_LIT(R, 1.0)));
        R sp, cp;
        m_sincos(phi, &sp, &cp);
        ps.dir = normalize3(ps.nrm + v3<R>(cp * cosTheta, sp * cosTheta, sinTheta));
    }
    ps.brdfPdf = dot3(ps.dir, ps.nrm) / PT_PI_R(R);
    const R numLights = S.numObjects[6];
    int pick = 0;
    uint32_t shadowState = 0;
    bool shadow = false;
    if (numLights > PT_LIT(R, 0.0)) {
        R boundingRadius = PT_LIT(R, 0.0);
        V3<R> lightPos = v3<R>(PT_LIT(R, 0.0), PT_LIT(R, 0.0), PT_LIT(R, 0.0));
        ps.shLightID = -PT_LIT(R, 1.0);
        ps.shObj = sample_random_light(S, ps.seed, boundingRadius, lightPos, ps.shLightID, pick);
        const R invLightDistance = PT_LIT(R, 1.0) / length3(lightPos - ps.org);
        const V3<R> lightDir = (lightPos - ps.org) * invLightDistance;
        const R sinthetaMax = m_fmin(boundingRadius * invLightDistance, PT_LIT(R, 1.0));
        const R costhetaMax = m_sqrt(PT_LIT(R, 1.0) - sinthetaMax * sinthetaMax);
        {  // SampleCosineUnitCone, SC:1012-1023.
            const R rx = rnd<R>(ps.seed);
            const R ry = rnd<R>(ps.seed);
            const R cosAlphaMax = PT_LIT(R, 2.0) * costhetaMax * costhetaMax - PT_LIT(R, 1.0);
            const R phi = PT_LIT(R, 2.0) * PT_PI_R(R) * ry;
            const R cosTheta = (PT_LIT(R, 1.0) - cosAlphaMax) * rx + cosAlphaMax;
            const R sinTheta = m_sqrt(m_fma(-cosTheta, cosTheta, PT_LIT(R, 1.0)));
            R sp, cp;
            m_sincos(phi, &sp, &cp);
            ps.shDir = to_world(normalize3(v3<R>(cp * sinTheta, sp * sinTheta, cosTheta + PT_LIT(R, 1.0))), lightDir);
        }
        ps.lightPdf = PT_LIT(R, 1.0) / numLights;
        ps.lightPdf *= dot3(ps.shDir, lightDir) / (PT_PI_R(R) * (PT_LIT(R, 1.0) - costhetaMax * costhetaMax));
        ps.mis = ps.brdfPdf * ps.brdfPdf / (ps.brdfPdf * ps.brdfPdf + ps.lightPdf * ps.lightPdf);
        ps.cosL = dot3(ps.shDir, ps.nrm);
        const R deathProbability = PT_LIT(R, 1.25) * m_fmax(ps.mis - PT_LIT(R, 0.2), PT_LIT(R, 0.0));
        if (ps.cosL >= PT_LIT(R, 0.0)) {
            if (rnd<R>(ps.seed) > deathProbability) {
                shadow = true;
            } else {
                ps.mis = PT_LIT(R, 1.0);
                shadowState = 1;
            }
        }
    } else {
        ps.mis = ps.brdfPdf * ps.brdfPdf / (ps.brdfPdf * ps.brdfPdf + PT_LIT(R, 0.0) * PT_LIT(R, 0.0));
    }
    if (TRACE) ps.ev |= ((uint32_t)(pick & 0x7F) << PT_EV_LIGHT_SHIFT) | (shadowState << PT_EV_SHADOW_SHIFT);
    if (shadow) return STEP_SHADOW;
    ps.radiance = ps.radiance + v4s<R>(PT_LIT(R, 0.0));
    return finish_bounce<TRACE>(ps, depth);
}

// The NEE term of a light sample whose shadow ray reached the light.
template <typename R> PT_DI V4<R> shadow_contribution(const PathStateT<R>& ps, const KScene& S) {
    const V2<R> lt = light_mix(S, ps.shLightID);
    const V4<R> rrl = ps.rr * ((ps.brdf * ps.cosL) / ps.lightPdf);
    return (emit(ps.l, lt.x, lt.y) * rrl) * (PT_LIT(R, 1.0) - ps.mis);
}

// LightSourceVisibilityCheck result (SC:1121-1223) and the NEE term, then the
// rest of the bounce.
template <bool TRACE, typename R>
PT_DI StepResult shade_shadow(PathStateT<R>& ps, const KScene& S, int objectID, int depth) {
    const int obj = (objectID == -2) ? -1 : objectID;
    V4<R> contrib = v4s<R>(PT_LIT(R, 0.0));
    if (obj == ps.shObj) {
        contrib = shadow_contribution(ps, S);
        if (TRACE) ps.ev |= 3u << PT_EV_SHADOW_SHIFT;
    } else {
        if (TRACE) ps.ev |= 2u << PT_EV_SHADOW_SHIFT;
    }
    ps.radiance = ps.radiance + contrib;
    return finish_bounce<TRACE>(ps, depth);
}

// shade_shadow with its two products made when the shadow ray was: the NEE
// term (shadow_contribution) and the bounce's next throughput
// (bounce_throughput), from the same values by the same operations, so the
// result is shade_shadow's bit for bit.  The staged engine stores those two
// instead of the light sample's geometry and the BRDF they come from.
template <bool TRACE, typename R>
PT_DI StepResult shade_shadow_made(PathStateT<R>& ps, int objectID, const V4<R>& contrib, const V4<R>& rr_next,
                                   int depth) {
    const int obj = (objectID == -2) ? -1 : objectID;
    V4<R> c = v4s<R>(PT_LIT(R, 0.0));
    if (obj == ps.shObj) {
        c = contrib;
        if (TRACE) ps.ev |= 3u << PT_EV_SHADOW_SHIFT;
    } else {
        if (TRACE) ps.ev |= 2u << PT_EV_SHADOW_SHIFT;
    }
    ps.radiance = ps.radiance + c;
    ps.rr = rr_next;
    return roulette<TRACE>(ps, depth);
}

// SC:1477-1489: the sample's XYZ with NaN rejection.
template <typename R> PT_DI V3<R> sample_color(const PathStateT<R>& ps, const KScene& S, const float* __restrict__ cie) {
    V3<R> wx, wy, wz, ww;
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
    const R range = (S.ext.flags & PT_EXT_WAVELENGTHS) ? (S.ext.lambda_max - S.ext.lambda_min) : (PT_LIT(R, 720.0) - PT_LIT(R, 390.0));
    V3<R> color = (((wx * ps.radiance.x + wy * ps.radiance.y) + wz * ps.radiance.z) + ww * ps.radiance.w) * range *
                   PT_LIT(R, 0.25);
    if (color.x != color.x || color.y != color.y || color.z != color.z) color = v3<R>(PT_LIT(R, 0.0), PT_LIT(R, 0.0), PT_LIT(R, 0.0));
    return color;
}

// Rendering + Accumulate, SC:1513-1520, SC:1492-1507: the pixel's new value
// from the ordered sample sum and the old accumulator value.
template <typename R = float> PT_DI V4<R> accumulate(const pt_push& pc, V3<R> sum, V4<R> old) {
    const R fs = (R)pc.samplesPerFrame;
    V3<R> out = v3<R>(sum.x / fs, sum.y / fs, sum.z / fs);
    out = out * (pc.apertureSize * pc.apertureSize * (R)pc.ISO);
    const V3<R> in = v3<R>(old.x, old.y, old.z);
    if ((pc.currentSamples == pc.samplesPerFrame) && (pc.frame > pc.samplesPerFrame)) {
        const R w = m_pow(PT_LIT(R, 2.0), -PT_LIT(R, 8.0) / (pc.FPS * pc.persistence));
        out = out * (PT_LIT(R, 1.0) - w) + in * w;
    } else {
        const int unitSamples = pc.currentSamples / pc.samplesPerFrame;
        const R us = (R)unitSamples;
        const V3<R> t = in * (R)(unitSamples - 1) + out;
        out = v3<R>(t.x / us, t.y / us, t.z / us);
    }
    return v4<R>(out.x, out.y, out.z, PT_LIT(R, 1.0));
}
