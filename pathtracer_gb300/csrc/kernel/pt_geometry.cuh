// pt_geometry.cuh — analytic primitives, SDF plug-ins and sphere tracing.
//
// Each function restates the cited lines of src/shader.comp (SC) with the
// same operation order; the differences are GPU-side only: rotation matrices
// come from the per-upload table (KScene::rot) and objects are read straight
// from the launch's constant bank instead of being unpacked into structs.
#pragma once

#include "pt_features.h"
#include "pt_scene.cuh"

#define PT_PI 3.141592653589792623810034526344f  // SC:9
#define PT_ONEBYTHREE 0.3333333f                 // SC:10
#define PT_MAXDIST 1e5f                          // SC:8

struct Hit {
    float hitdist;
    float3 normal;
    float materialID;
    float lightID;
};

// BoundingSphere, SC:263-276.
PT_DI bool bounding_sphere(float3 org, float3 dir, float3 pos, float radius2) {
    const float3 lo = org - pos;
    const float b = dot3(dir, lo);
    const float c = dot3(lo, lo) - radius2;
    if ((b * b) < c) return false;
    if ((b >= 0.0f) && (c >= 0.0f)) return false;
    return true;
}

// SphereIntersection, SC:289-317.
PT_DI bool sphere_intersect(float3 org, float3 dir, float3 pos, float radius, float mat, float light, Hit& h) {
    const float3 lo = org - pos;
    const float b = 2.0f * dot3(dir, lo);
    const float c = dot3(lo, lo) - (radius * radius);
    const float disc = b * b - 4.0f * c;
    if (disc < 0.0f) return false;
    const float sqrtD = sqrtf(disc);
    const float t1 = (-b - sqrtD) * 0.5f;
    const float t2 = (-b + sqrtD) * 0.5f;
    const float t = (t1 > 0.0f) ? t1 : t2;
    const float isOutside = (t1 > 0.0f) ? 1.0f : -1.0f;
    if (t < 1e-4f) return false;
    if (t < h.hitdist) {
        h.hitdist = t;
        h.normal = normalize3(fma3s(dir, t, lo) * isOutside);
        h.materialID = mat;
        h.lightID = light;
        return true;
    }
    return false;
}

// PlaneIntersection, SC:319-335.
PT_DI bool plane_intersect(float3 org, float3 dir, float3 pos, float mat, float light, Hit& h) {
    const float3 lo = org - pos;
    const float t = -lo.y / dir.y;
    if (t < 1e-4f) return false;
    if (t < h.hitdist) {
        h.hitdist = t;
        const float d = 0.0f * dir.x + 1.0f * dir.y + 0.0f * dir.z;  // faceforward: dot(Nref, I)
        h.normal = (d < 0.0f) ? f3(0.0f, 1.0f, 0.0f) : f3(-0.0f, -1.0f, -0.0f);
        h.materialID = mat;
        h.lightID = light;
        return true;
    }
    return false;
}

// BoxIntersection, SC:337-364 (matrix from KScene::rot).
PT_DI bool box_intersect(float3 org, float3 dir_w, float3 pos, float3 size, const m3& m, float mat, float light, Hit& h) {
    const float3 lo = mul_vm(org - pos, m);
    const float3 dir = mul_vm(dir_w, m);
    const float3 invdir = f3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    const float3 tMin0 = fma3(size, f3(-0.5f, -0.5f, -0.5f), -lo) * invdir;
    const float3 tMax0 = fma3(size, f3(0.5f, 0.5f, 0.5f), -lo) * invdir;
    const float3 a = min3(tMin0, tMax0), bb = max3(tMin0, tMax0);
    const float t1 = fmaxf(fmaxf(a.x, a.y), a.z);
    const float t2 = fminf(fminf(bb.x, bb.y), bb.z);
    const float t = (t1 < 0.0f) ? t2 : t1;
    if ((t1 > t2) || (t < 1e-4f)) return false;
    if (t < h.hitdist) {
        h.hitdist = t;
        const float3 p = abs3((lo + dir * t) / size);
        const float mx = fmaxf(fmaxf(p.x, p.y), p.z);
        const float3 st = f3(step_glsl(mx, p.x), step_glsl(mx, p.y), step_glsl(mx, p.z));
        const float3 sg = f3(-sign_glsl(dir.x), -sign_glsl(dir.y), -sign_glsl(dir.z));
        h.normal = mul_mv(m, st * sg);
        h.materialID = mat;
        h.lightID = light;
        return true;
    }
    return false;
}

// Lens geometry shared by the camera lens and scene lenses.
struct LensGeom {
    float3 pos;
    m3 rot;
    float radius;        // lens aperture radius
    float focal;         // focal length
    float thickness;
    bool converging;
};

// SphereSliceIntersection, SC:366-417.
PT_DI bool slice_intersect(float3 org_w, float3 dir_w, const LensGeom& L, float sliceRadius, float sliceSize,
                           bool is1st, float localSlicePos, bool isSideInvert, float mat, float light, Hit& h,
                           int& isOutside) {
    const float sliceOffset = sliceRadius - sliceSize;
    float3 org = mul_vm(org_w - L.pos, L.rot);
    if (is1st) {
        org.x += localSlicePos - sliceSize - sliceOffset;
    } else {
        org.x -= localSlicePos - sliceSize - sliceOffset;
    }
    const float3 dir = mul_vm(dir_w, L.rot);
    const float b = 2.0f * dot3(dir, org);
    const float c = dot3(org, org) - (sliceRadius * sliceRadius);
    const float disc = b * b - 4.0f * c;
    float t = 1e6f;
    int isOut = 1;
    if (disc < 0.0f) return false;
    const float sqrtD = sqrtf(disc);
    float t1 = (-b - sqrtD) * 0.5f;
    float t2 = (-b + sqrtD) * 0.5f;
    if (is1st) {
        t1 = (__fmaf_rn(dir.x, t1, org.x) > -sliceOffset) ? 1e6f : t1;
        t2 = (__fmaf_rn(dir.x, t2, org.x) > -sliceOffset) ? 1e6f : t2;
    } else {
        t1 = (__fmaf_rn(dir.x, t1, org.x) < sliceOffset) ? 1e6f : t1;
        t2 = (__fmaf_rn(dir.x, t2, org.x) < sliceOffset) ? 1e6f : t2;
    }
    t = (t1 > 0.0f) ? t1 : t;
    if (t2 < t) {
        t = t2;
        isOut = -1;
    }
    if (t < 1e-4f) return false;
    if (t < h.hitdist) {
        h.hitdist = t;
        h.normal = mul_mv(L.rot, normalize3(fma3s(dir, t, org) * (float)isOut));
        isOutside = (!isSideInvert) ? isOut : -isOut;
        h.materialID = mat;
        h.lightID = light;
        return true;
    }
    return false;
}

// LensIntersection, SC:419-448.
PT_DI bool lens_intersect(float3 org, float3 dir, const LensGeom& L, float mat, float light, Hit& h, int& isOutside) {
    const float lensThicknessHalf = 2.0f * L.focal - sqrtf(4.0f * L.focal * L.focal - L.radius * L.radius);
    float lensSlicePos = 0.5f * (L.converging ? L.thickness : -L.thickness);
    if (L.converging) lensSlicePos += lensThicknessHalf;
    const float sliceRadius = 2.0f * L.focal;
    bool hit = false;
#pragma unroll
    for (int i = 0; i < 2; i++) {
        if (slice_intersect(org, dir, L, sliceRadius, lensThicknessHalf, i == 0, lensSlicePos, !L.converging, mat,
                            light, h, isOutside))
            hit = true;
    }
    return hit;
}

PT_DI float lens_bounding_radius2(float radius, float focal, float thickness, bool converging) {
    float br;
    if (converging) {
        br = (radius * radius) + (0.25f * thickness * thickness);
    } else {
        br = 0.5f * thickness + 2.0f * focal - sqrtf(4.0f * focal * focal - radius * radius);
        br = br * br + radius * radius;
    }
    return br;
}

// ---------------------------------------------------------------------------
// Quartic / cubic solvers (SC:450-541) and the Dupin cyclide (SC:633-679).
PT_DI float eval_quadratic(float a, float b, float c, float x) { return x * (x * a + b) + c; }
PT_DI float eval_cubic(float a, float b, float c, float d, float x) { return x * (x * (x * a + b) + c) + d; }
PT_DI float eval_quartic(float a, float b, float c, float d, float e, float x) {
    return x * (x * (x * (x * a + b) + c) + d) + e;
}

// SolveCubic, SC:474-503; only the first root is consumed by SolveQuartic.
PT_DI float solve_cubic_first(float b, float c, float d) {
    const float bdiv3 = b * PT_ONEBYTHREE;
    const float Q = c * PT_ONEBYTHREE - bdiv3 * bdiv3;
    const float R = 0.5f * bdiv3 * c - bdiv3 * bdiv3 * bdiv3 - 0.5f * d;
    const float D = Q * Q * Q + R * R;
    float x;
    if (D > 0.0f) {
        const float u = R + sqrtf(D);
        const float v = R - sqrtf(D);
        const float S = sign_glsl(u) * ptm_powf(fabsf(u), PT_ONEBYTHREE);
        const float T = sign_glsl(v) * ptm_powf(fabsf(v), PT_ONEBYTHREE);
        x = S + T - bdiv3;
    } else {
        const float sqrtnegQ = sqrtf(-Q);
        const float thetadiv3 = ptm_acosf(R / (sqrtnegQ * sqrtnegQ * sqrtnegQ)) * PT_ONEBYTHREE;
        x = 2.0f * sqrtnegQ * ptm_cosf(thetadiv3) - bdiv3;
    }
#pragma unroll
    for (int i = 0; i < 2; i++) x -= eval_cubic(1.0f, b, c, d, x) / eval_quadratic(3.0f, 2.0f * b, c, x);
    return x;
}

// SolveQuartic, SC:505-541, folded into "smallest positive real root below t".
PT_DI float solve_quartic_min_positive(float a, float b, float c, float d, float e) {
    const float inva = 1.0f / a;
    const float inva2 = inva * 0.5f;
    const float inva2a2 = inva2 * inva2;
    const float bb = b * b;
    const float p = -1.5f * bb * inva2a2 + c * inva;
    const float q = bb * b * inva2a2 * inva2 - b * c * inva * inva2 + d * inva;
    const float r = -0.1875f * bb * bb * inva2a2 * inva2a2 + 0.5f * c * bb * inva2a2 * inva2 - b * d * inva2a2 + e * inva;
    const float sx = solve_cubic_first(0.5f * -p, -r, 0.5f * p * r - 0.125f * q * q);
    float t = 1e6f;
    const float s2subp = 2.0f * sx - p;
    if (s2subp < 0.0f) return t;
    const float invs2subp = -2.0f * sx - p;
    const float sqrts2subp = sqrtf(s2subp);
    const float q2divsqrt = 2.0f * q / sqrts2subp;
    const float invaddq2div = invs2subp + q2divsqrt;
    const float invsubq2div = invs2subp - q2divsqrt;
    const float bdiv4a = 0.25f * inva * b;
    float r0 = 0.0f, r1 = 0.0f, r2 = 0.0f, r3 = 0.0f;
    const bool re01 = invaddq2div >= 0.0f;
    const bool re23 = invsubq2div >= 0.0f;
    if (re01) {
        const float sq = sqrtf(invaddq2div);
        r0 = 0.5f * (-sqrts2subp + 1.0f * sq) - bdiv4a;
        r1 = 0.5f * (-sqrts2subp + -1.0f * sq) - bdiv4a;
        r0 -= eval_quartic(a, b, c, d, e, r0) / eval_cubic(4.0f * a, 3.0f * b, 2.0f * c, d, r0);
        r1 -= eval_quartic(a, b, c, d, e, r1) / eval_cubic(4.0f * a, 3.0f * b, 2.0f * c, d, r1);
    }
    if (re23) {
        const float sq = sqrtf(invsubq2div);
        r2 = 0.5f * (sqrts2subp + 1.0f * sq) - bdiv4a;
        r3 = 0.5f * (sqrts2subp + -1.0f * sq) - bdiv4a;
        r2 -= eval_quartic(a, b, c, d, e, r2) / eval_cubic(4.0f * a, 3.0f * b, 2.0f * c, d, r2);
        r3 -= eval_quartic(a, b, c, d, e, r3) / eval_cubic(4.0f * a, 3.0f * b, 2.0f * c, d, r3);
    }
    // DupinCyclide SC:648-655: scan the real roots in order.
    if (re01) {
        if ((r0 < t) && (r0 > 0.0f)) t = r0;
        if ((r1 < t) && (r1 > 0.0f)) t = r1;
    }
    if (re23) {
        if ((r2 < t) && (r2 > 0.0f)) t = r2;
        if ((r3 < t) && (r3 > 0.0f)) t = r3;
    }
    return t;
}

PT_DI float3 sw_xzy(float3 v) { return f3(v.x, v.z, v.y); }
PT_DI float3 sw_yzx(float3 v) { return f3(v.y, v.z, v.x); }
PT_DI float3 sw_zxy(float3 v) { return f3(v.z, v.x, v.y); }

// DupinCyclide, SC:633-679.  base = float offset of the cyclide in objects[].
PT_DI bool cyclide_intersect(const KScene& S, float3 org, float3 dir, int base, const m3& m, Hit& h) {
    const float3 pos = f3(S.objects[base], S.objects[base + 1], S.objects[base + 2]);
    const float3 scale = f3(S.objects[base + 6], S.objects[base + 7], S.objects[base + 8]);
    const float A = S.objects[base + 9], B = S.objects[base + 10];
    const float C = S.objects[base + 11], Dd = S.objects[base + 12];
    const float3 o = sw_xzy(mul_vm(org - pos, m) / scale);
    const float3 d = sw_xzy(mul_vm(dir, m) / scale);
    const float3 dd = d * d, oo = o * o, od = o * d;
    const float3 dyzx = sw_yzx(d), dzxy = sw_zxy(d), oyzx = sw_yzx(o), ozxy = sw_zxy(o);
    const float a4 = dot3(dd, dd) + 2.0f * dot3(dd, dyzx * dyzx);
    const float a3 = 4.0f * (dot3(o, dd * d) + dot3(od, dyzx * dyzx) + dot3(od, dzxy * dzxy));
    const float a2 = 6.0f * dot3(oo, dd) + 8.0f * dot3(od, oyzx * dyzx) +
                     2.0f * (dot3(oo, dyzx * dyzx) + dot3(oo, dzxy * dzxy)) + 2.0f * (B * B - Dd * Dd) * dot3(d, d) -
                     4.0f * (A * A * d.x * d.x + B * B * d.y * d.y);
    const float a1 = 4.0f * (dot3(oo * o, d) + dot3(oo, oyzx * dyzx) + dot3(oo, ozxy * dzxy) + 2.0f * A * C * Dd * d.x +
                             (B * B - Dd * Dd) * dot3(o, d) - 2.0f * (A * A * o.x * d.x + B * B * o.y * d.y));
    const float a0 = dot3(oo, oo) + 2.0f * dot3(oo, oyzx * oyzx) + B * B * B * B + Dd * Dd * Dd * Dd -
                     2.0f * B * B * Dd * Dd - 4.0f * C * C * Dd * Dd + 8.0f * A * C * Dd * o.x +
                     2.0f * (B * B - Dd * Dd) * dot3(o, o) - 4.0f * (A * A * o.x * o.x + B * B * o.y * o.y);
    const float t = solve_quartic_min_positive(a4, a3, a2, a1, a0);
    if (t < h.hitdist) {
        h.hitdist = t;
        const float x = o.x + d.x * t;
        const float y = o.y + d.y * t;
        const float z = o.z + d.z * t;
        const float term1 = x * x + y * y + z * z + B * B - Dd * Dd;
        const float3 n = f3(4.0f * (x * term1 - 2.0f * A * (A * x - C * Dd)), 4.0f * z * term1,
                            4.0f * y * (term1 - 2.0f * B * B));
        h.normal = normalize3(n);
        h.materialID = (float)((int)S.objects[base + 14] - 1);
        h.lightID = (float)((int)S.objects[base + 15] - 1);
        return true;
    }
    return false;
}

// The smallest positive real root of a4 t^4 + ... + a0 below 1e6 by the
// shader's SolveQuartic and root scan (SC:505-541 with the loop of SC:560-567).
// Thritorius, SC:543-588: a quartic surface at the origin in the ray's xzy
// frame.  The shader defines it and SmoothCuboid but comments out their call
// sites (SC:926-931, :1207-1216), so no scene reaches either; they are
// built for completeness and evaluated through pt_quartic_surface_eval.
PT_DI bool thritorius_intersect(float3 org, float3 dir, Hit& h) {
    if (!bounding_sphere(org, dir, f3(0.0f, 0.0f, 0.0f), 4.05f)) return false;
    const float3 o = sw_xzy(org), d = sw_xzy(dir);
    const float3 ddd = (d * d) * d;
    const float3 d10 = f3(d.x, d.y, 10.0f * d.z), o10 = f3(o.x, o.y, 10.0f * o.z);
    const float a4 = dot3(d10, ddd) + 2.0f * dot3(d * d, sw_yzx(d) * sw_yzx(d));
    const float3 dd2 = f3(d.y * d.y + d.z * d.z, d.x * d.x + d.z * d.z, d.x * d.x + d.y * d.y);
    const float a3 = 4.0f * (dot3(o10, ddd) + dot3(o * d, dd2)) + 2.0f * d.y * d.y * d.y - 6.0f * d.x * d.x * d.y;
    const float3 oxxy = f3(o.x, o.x, o.y), dxxy = f3(d.x, d.x, d.y), oyzz = f3(o.y, o.z, o.z), dyzz = f3(d.y, d.z, d.z);
    const float a2 = 6.0f * dot3(o10, (o * d) * d) +
                     2.0f * ((o.x * o.x * (d.y * d.y) + o.y * o.y * (d.x * d.x)) +
                             (o.x * o.x * (d.z * d.z) + o.z * o.z * (d.x * d.x)) +
                             (o.y * o.y * (d.z * d.z) + o.z * o.z * (d.y * d.y))) +
                     8.0f * dot3(oxxy * dxxy, oyzz * dyzz) + 6.0f * o.y * d.y * d.y - 6.0f * o.y * d.x * d.x -
                     12.0f * o.x * d.x * d.y - 12.0f * d.z * d.z;
    const float a1 = 4.0f * (dot3((o10 * o) * o, d) + (o.x * o.x * (o.y * d.y) + o.x * o.x * (o.z * d.z)) +
                             (o.y * o.y * (o.x * d.x) + o.y * o.y * (o.z * d.z)) +
                             (o.z * o.z * (o.x * d.x) + o.z * o.z * (o.y * d.y))) +
                     6.0f * o.y * o.y * d.y - 6.0f * o.x * o.x * d.y - 12.0f * o.x * o.y * d.x - 24.0f * o.z * d.z;
    const float a0 = dot3(o10, (o * o) * o) + 2.0f * dot3(oxxy * oxxy, oyzz * oyzz) + 2.0f * o.y * o.y * o.y -
                     6.0f * o.x * o.x * o.y - 12.0f * o.z * o.z + 1.0f;
    const float t = solve_quartic_min_positive(a4, a3, a2, a1, a0);
    if (t < h.hitdist) {
        h.hitdist = t;
        const float x = o.x + d.x * t;
        const float y = o.y + d.y * t;
        const float z = o.z + d.z * t;
        float3 n = f3(4.0f * x * x * x + 4.0f * x * y * y - 12.0f * x * y + 4.0f * x * z * z,
                      40.0f * z * z * z + 4.0f * x * x * z + 4.0f * y * y * z - 24.0f * z,
                      4.0f * y * y * y + 4.0f * x * x * y - 6.0f * x * x + 6.0f * y * y + 4.0f * y * z * z);
        if ((o.x * o.x * (o.x * o.x + 2.0f * o.y * o.y - 6.0f * o.y + 2.0f * o.z * o.z) +
             o.y * o.y * (o.y * o.y + 2.0f * o.y + 2.0f * o.z * o.z) + o.z * o.z * (10.0f * o.z * o.z - 12.0f) +
             1.0f) < 0.0f)
            n = n * -1.0f;
        h.normal = normalize3(n);
        h.materialID = 1.0f;
        h.lightID = -1.0f;
        return true;
    }
    return false;
}

// SmoothCuboid, SC:590-631: x^4 + y^4 + z^4 = 1 at the origin.
PT_DI bool smooth_cuboid_intersect(float3 o, float3 d, Hit& h) {
    if (!bounding_sphere(o, d, f3(0.0f, 0.0f, 0.0f), 1.80f)) return false;
    const float a4 = dot3(d * d, d * d);
    const float a3 = 4.0f * dot3(o, (d * d) * d);
    const float a2 = 6.0f * dot3(o * o, d * d);
    const float a1 = 4.0f * dot3((o * o) * o, d);
    const float a0 = dot3(o * o, o * o) - 1.0f;
    const float t = solve_quartic_min_positive(a4, a3, a2, a1, a0);
    if (t < h.hitdist) {
        h.hitdist = t;
        float3 n = fma3s(d, t, o);
        n = (n * n) * n;
        if (dot3(o * o, o * o) < 1.0f) n = n * -1.0f;
        h.normal = normalize3(n);
        h.materialID = 3.0f;
        h.lightID = -1.0f;
        return true;
    }
    return false;
}

// ---------------------------------------------------------------------------
// SDF plug-ins: the four snippets of sdfs/<name>.glsl as __device__ functions
// with the snippets' signature `float sdf(vec3 p)` / `float sdfmaterial(vec3 p)`.

// smin, SC:686-702.
PT_DI float smin1(float x, float y) {
    float k = 0.02f;
    k *= 6.0f;
    const float h = fmaxf(k - fabsf(x - y), 0.0f) / k;
    const float m = h * h * h * 0.5f;
    const float s = m * k * PT_ONEBYTHREE;
    return fminf(x, y) - s;
}
PT_DI float2 smin2(float2 x, float2 y) {
    float k = 0.02f;
    k *= 6.0f;
    const float h = fmaxf(k - fabsf(x.x - y.x), 0.0f) / k;
    const float m = h * h * h * 0.5f;
    const float s = m * k * PT_ONEBYTHREE;
    return (x.x < y.x) ? make_float2(x.x - s, x.y + (y.y - x.y) * m)
                       : make_float2(y.x - s, x.y + (y.y - x.y) * (1.0f - m));
}

namespace sdf_blob {  // sdfs/blob.glsl
PT_DI float sdf(float3 p) {
    const float s1 = length3(p) - 1.0f;
    const float s2 = length3(f3(p.x, p.y - 1.0f, p.z)) - 0.7f;
    const float s3 = length3(f3(p.x - 0.25f, p.y - 1.25f, p.z - 0.5f)) - 0.25f;
    const float s4 = length3(f3(p.x + 0.25f, p.y - 1.25f, p.z - 0.5f)) - 0.25f;
    return smin1(smin1(smin1(s1, s2), s3), s4);
}
PT_DI float sdfmaterial(float3 p, const float* m) {
    const float2 s1 = make_float2(length3(p) - 1.0f, m[0]);
    const float2 s2 = make_float2(length3(f3(p.x, p.y - 1.0f, p.z)) - 0.7f, m[1]);
    const float2 s3 = make_float2(length3(f3(p.x - 0.25f, p.y - 1.25f, p.z - 0.5f)) - 0.25f, m[2]);
    const float2 s4 = make_float2(length3(f3(p.x + 0.25f, p.y - 1.25f, p.z - 0.5f)) - 0.25f, m[2]);
    return smin2(smin2(smin2(s1, s2), s3), s4).y;
}
}  // namespace sdf_blob

namespace sdf_mandelbulb {  // sdfs/mandelbulb.glsl (power 8, 4 iterations, bailout 16)
PT_DI float sdf(float3 p) {
    float3 z = p;
    float r = length3(z);
    float dr = 1.0f;
#pragma unroll 1
    for (int i = 0; i < 4; i++) {
        dr = 8.0f * pow_pos_int<7>(r) * dr + 1.0f;  // r = length(z): +0, positive, +inf or NaN
        const float invr = 1.0f / r;
        const float invl = 1.0f / sqrtf(z.x * z.x + z.z * z.z);
        r *= r;
        r *= r;
        r *= r;
        const float cost = z.z * invl;
        const float cosp = z.y * invr;
        const float sint = z.x * invl;
        const float sinp = invr / invl;
        const float cost2 = cost * cost;
        const float cosp2 = cosp * cosp;
        const float cost8 =
            __fmaf_rn(__fmaf_rn(__fmaf_rn(__fmaf_rn(128.0f, cost2, -256.0f), cost2, 160.0f), cost2, -32.0f), cost2, 1.0f);
        const float cosp8 =
            __fmaf_rn(__fmaf_rn(__fmaf_rn(__fmaf_rn(128.0f, cosp2, -256.0f), cosp2, 160.0f), cosp2, -32.0f), cosp2, 1.0f);
        const float sint8 = __fmaf_rn(__fmaf_rn(__fmaf_rn(128.0f, cost2, -192.0f), cost2, 80.0f), cost2, -8.0f) * sint * cost;
        const float sinp8 = __fmaf_rn(__fmaf_rn(__fmaf_rn(128.0f, cosp2, -192.0f), cosp2, 80.0f), cosp2, -8.0f) * sinp * cosp;
        z = f3(sint8 * sinp8, cosp8, cost8 * sinp8) * r;
        z = z + p;
        r = length3(z);
        if (r > 16.0f) break;
    }
    return 0.5f * ptm_logf_inline(r) * r / dr;  // inlined: the march loop's hottest call
}
PT_DI float sdfmaterial(float3 p, const float* m) {
    const float factor = dot3(p, p);
    return mix_glsl(m[0], m[1], factor / (0.8f + factor));
}
}  // namespace sdf_mandelbulb

namespace sdf_menger {  // sdfs/menger.glsl
PT_DI float sdf(float3 p) {
    const float3 q = abs3(p) - f3(1.0f, 1.0f, 1.0f);
    float d = length3(max3(q, f3(0.0f, 0.0f, 0.0f))) + fminf(fmaxf(q.x, fmaxf(q.y, q.z)), 0.0f);
    float s = 1.0f;
#pragma unroll 1
    for (int m = 0; m < 5; m++) {
        const float3 ps = p * s;
        const float3 a = f3(mod_glsl(ps.x, 2.0f) - 1.0f, mod_glsl(ps.y, 2.0f) - 1.0f, mod_glsl(ps.z, 2.0f) - 1.0f);
        s *= 3.0f;
        const float3 r =
            f3(fabsf(1.0f - 3.0f * fabsf(a.x)), fabsf(1.0f - 3.0f * fabsf(a.y)), fabsf(1.0f - 3.0f * fabsf(a.z)));
        const float da = fmaxf(r.x, r.y);
        const float db = fmaxf(r.y, r.z);
        const float dc = fmaxf(r.z, r.x);
        const float c = (fminf(da, fminf(db, dc)) - 1.0f) / s;
        d = fmaxf(d, c);
    }
    return d;
}
}  // namespace sdf_menger

namespace sdf_terrain {  // sdfs/terrain.glsl
PT_DI float height(float x) {
    return ptm_sinf_inline(0.0625f * x) + ptm_sinf_inline(0.125f * (x + 10.0f)) + 0.25f * ptm_sinf_inline(0.25f * x) + 0.125f * ptm_sinf_inline(0.5f * x) +
           0.25f * ptm_sinf_inline(x) + 0.25f * ptm_sinf_inline(2.0f * x + 1.0f) + 0.125f * ptm_sinf_inline(4.0f * x + 2.0f) +
           0.0625f * ptm_sinf_inline(8.0f * x + 1.0f) + 0.03125f * ptm_sinf_inline(16.0f * x + 5.0f) + 0.015625f * ptm_sinf_inline(32.0f * x) +
           0.0078125f * ptm_sinf_inline(64.0f * x);
}
PT_DI float sdf(float3 p) { return p.y - (height(p.x) + height(p.z)); }
}  // namespace sdf_terrain

// A scene's SDF slot `slot` with plug-in `kind`.  PT_SDF_CUSTOM slots hold
// GLSL compiled at run time: the module built for them (pt_jit.cu) defines
// pt_user_sdf / pt_user_material before including these headers; the
// precompiled kernels never see that kind.
PT_DI float plugin_sdf(int kind, int slot, float3 p) {
    switch (kind) {
        case PT_SDF_MANDELBULB: return sdf_mandelbulb::sdf(p);
        case PT_SDF_MENGER: return sdf_menger::sdf(p);
        case PT_SDF_BLOB: return sdf_blob::sdf(p);
        case PT_SDF_TERRAIN: return sdf_terrain::sdf(p);
#if defined(PT_JIT_USER_SDF)
        case PT_SDF_CUSTOM: return pt_user_sdf(slot, p);
#endif
        default: return PT_MAXDIST;
    }
}
PT_DI float plugin_material(const pt_sdf_plugin& pl, int slot, float3 p) {
    if (pl.material_mode == PT_SDFMAT_CONSTANT) return pl.material[0];
    switch (pl.kind) {
        case PT_SDF_BLOB: return sdf_blob::sdfmaterial(p, pl.material);
        case PT_SDF_MANDELBULB: return sdf_mandelbulb::sdfmaterial(p, pl.material);
#if defined(PT_JIT_USER_SDF)
        case PT_SDF_CUSTOM: return pt_user_material(slot, p);
#endif
        default: return pl.material[0];
    }
}
PT_DI float3 sdf_pos(const KScene& S, int i) { return f3(S.sdfs[6 * i], S.sdfs[6 * i + 1], S.sdfs[6 * i + 2]); }

// SDF() with the lines InsertSDF splices in (src/pathtracer.cpp:2004-2054):
// in scene order, sdf = min(sdf, SDFi(p - pos_i)) for every bit i of set1.
PT_DI float scene_sdf(const KScene& S, float3 p, uint32_t set1) {
    float sdf = PT_MAXDIST;
    uint32_t bits = set1 & ((S.meta.nplug >= 32) ? 0xFFFFFFFFu : ((1u << S.meta.nplug) - 1u));
    while (bits) {
        const int i = __ffs(bits) - 1;
        bits &= bits - 1u;
        const int kind = S.plug[i].kind;
        if (kind != PT_SDF_NONE) sdf = fminf(sdf, plugin_sdf(kind, S.meta.custom_base + i, p - sdf_pos(S, i)));
    }
    return sdf;
}
// scene_sdf that also reports the SDF whose material SDFMATERIAL() picks at
// p (SC:713-719: the last i with !(running minimum < d_i); -1 for none), so
// a march that converged at p needs only that SDF's material function there.
PT_DI float scene_sdf_sel(const KScene& S, float3 p, uint32_t set1, int& sel) {
    float sdf = PT_MAXDIST;
    sel = -1;
    uint32_t bits = set1 & ((S.meta.nplug >= 32) ? 0xFFFFFFFFu : ((1u << S.meta.nplug) - 1u));
    while (bits) {
        const int i = __ffs(bits) - 1;
        bits &= bits - 1u;
        const int kind = S.plug[i].kind;
        if (kind != PT_SDF_NONE) {
            const float di = plugin_sdf(kind, S.meta.custom_base + i, p - sdf_pos(S, i));
            if (!(sdf < di)) sel = i;
            sdf = fminf(sdf, di);
        }
    }
    return sdf;
}
// Out-of-line copy for the cold call sites (sign at the origin, normals).
static __device__ __noinline__ float scene_sdf_cold(const KScene& S, float3 p, uint32_t set1) { return scene_sdf(S, p, set1); }

// SDFMATERIAL() with the spliced minMaterial lines (SC:681-683, SC:713-719).
static __device__ __noinline__ float scene_sdf_material(const KScene& S, float3 p, uint32_t set1) {
    float sdf = PT_MAXDIST;
    float mat = 0.0f;
    uint32_t bits = set1 & ((S.meta.nplug >= 32) ? 0xFFFFFFFFu : ((1u << S.meta.nplug) - 1u));
    while (bits) {
        const int i = __ffs(bits) - 1;
        bits &= bits - 1u;
        const pt_sdf_plugin pl = S.plug[i];
        if (pl.kind != PT_SDF_NONE) {
            const float3 q = p - sdf_pos(S, i);
            const float di = plugin_sdf(pl.kind, S.meta.custom_base + i, q);
            mat = (sdf < di) ? mat : plugin_material(pl, S.meta.custom_base + i, q);
            sdf = fminf(sdf, di);
        }
    }
    return mat;
}

// SDFMATERIAL (SC:704-719) at a sphere-tracing hit p.  hit_sel >= -1: the
// march converged on an evaluation at p itself, and hit_sel is what
// scene_sdf_sel reported there (the same distances in the same order), so the
// reference's selection reduces to that SDF's sdfmaterial at p, or 0 for
// none, without evaluating the distances again; otherwise (-2: the march ran
// out of steps) the full selection runs.
PT_DI float scene_sdf_material_hit(const KScene& S, float3 p, uint32_t set1, int hit_sel) {
    if (hit_sel >= 0) return plugin_material(S.plug[hit_sel], S.meta.custom_base + hit_sel, p - sdf_pos(S, hit_sel));
    if (hit_sel == -1) return 0.0f;
    return scene_sdf_material(S, p, set1);
}

// RayIntersectAABB, SC:278-287.
PT_DI float2 ray_aabb(float3 origin, float3 invdir, float3 pos, float3 size) {
    const float3 lo = origin - pos;
    const float3 tMin0 = fma3(size, f3(-0.5f, -0.5f, -0.5f), -lo) * invdir;
    const float3 tMax0 = fma3(size, f3(0.5f, 0.5f, 0.5f), -lo) * invdir;
    const float3 a = min3(tMin0, tMax0), b = max3(tMin0, tMax0);
    return make_float2(fmaxf(fmaxf(a.x, a.y), a.z), fminf(fminf(b.x, b.y), b.z));
}

// SearchSDF, SC:732-777.
PT_DI bool search_sdf(const KScene& S, float3 p, float3 invdir, float2& tMinMax, uint32_t& set1) {
    bool found = false;
    set1 = 0;
    const int n = S.meta.n[5];
    for (int i = 0; i < n; i++) {
        const float3 pos = sdf_pos(S, i);
        const float3 size = f3(S.sdfs[6 * i + 3], S.sdfs[6 * i + 4], S.sdfs[6 * i + 5]);
        const float2 bm = ray_aabb(p, invdir, pos, size);
        const uint32_t bit = 1u << i;  // n <= 32 is enforced on upload
        if ((bm.x > bm.y) || (bm.y < 0.0f)) continue;
        if (bm.x < tMinMax.x) {
            found = true;
            if (bm.y < tMinMax.x) {
                tMinMax = bm;
                set1 = bit;
            } else if (bm.y < tMinMax.y) {
                tMinMax.x = bm.x;
                set1 += bit;
            } else {
                tMinMax = bm;
                set1 += bit;
            }
        } else if (bm.x < tMinMax.y) {
            found = true;
            if (bm.y > tMinMax.y) tMinMax.y = bm.y;
            set1 += bit;
        }
    }
    return found;
}

// SphereTracing, SC:779-860.  Returns true when it replaced the hit.
PT_DI bool sphere_trace(const KScene& S, float3 org, float3 dir, Hit& h) {
    float t = 1e-3f;
    float insT = 0.0f;
    const float omegaMax = 1.70f;
    const float omegaSpeed = 0.20f;
    float omega = omegaMax;
    float previousRadius = 0.0f;
    const float3 invdir = f3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
    int points = 0;
    float2 tMinMax = make_float2(PT_MAXDIST, PT_MAXDIST);
    uint32_t set1 = 0;
    float3 p;
    if (search_sdf(S, org, invdir, tMinMax, set1)) {
        t = fmaxf(tMinMax.x, t);
        p = fma3s(dir, t, org);
    } else {
        return false;
    }
    const float k = sign_glsl(scene_sdf_cold(S, org, set1));
    int hit_sel = -2;  // >= -1 once the march converged (scene_sdf_material_hit)
    // The reference's limits (512 steps, |d| < 1e-4, no distance cap) or the
    // scene's PT_EXT_MARCH ones.
    const bool xm = (S.ext.flags & PT_EXT_MARCH) != 0;
    const int maxSteps = xm ? S.ext.march_max_steps : 512;
    const float eps = xm ? S.ext.march_epsilon : 1e-4f;
    const float tmax = xm ? S.ext.march_max_distance : __int_as_float(0x7f800000);
#pragma unroll 1
    for (int i = 0; i < maxSteps; i++) {
        if (t > tmax) return false;  // past the distance cap: no SDF hit
        int sel;
        const float radius = scene_sdf_sel(S, p, set1, sel);
        if (insT > (fabsf(previousRadius) + fabsf(radius))) {
            t -= insT;
            omega = 1.0f;
            insT = previousRadius * omega * k;
            t += insT;
            p = fma3s(dir, t, org);
            continue;
        }
        if (fabsf(radius) < eps) {
            hit_sel = sel;
            break;
        }
        if (t > tMinMax.y) {
            points += 1;
        } else {
            points = 0;
        }
        if (points >= 2) {
            t = tMinMax.y + 1e-3f;
            tMinMax = make_float2(PT_MAXDIST, PT_MAXDIST);
            if (search_sdf(S, fma3s(dir, t, org), invdir, tMinMax, set1)) {
                tMinMax.x += t;
                tMinMax.y += t;
                t = fmaxf(tMinMax.x, t);
                p = fma3s(dir, t, org);
                continue;
            }
            return false;
        }
        insT = radius * omega * k;
        t += insT;
        p = fma3s(dir, t, org);
        const float omegaSpeedFactor = fminf(radius / previousRadius, 0.99f);
        omega += omegaSpeed * (fminf(1.0f / (1.0f - omegaSpeedFactor), omegaMax) - omega);
        previousRadius = radius;
    }
    if (t < h.hitdist) {
        h.hitdist = t - 1e-3f;
        p = fma3s(dir, t, org);
        // CalculateNumericalSDFNormals, SC:721-730.
        const float e = 1e-4f;
        const float nx = scene_sdf_cold(S, f3(p.x + e, p.y + 0.0f, p.z + 0.0f), set1) -
                         scene_sdf_cold(S, f3(p.x - e, p.y - 0.0f, p.z - 0.0f), set1);
        const float ny = scene_sdf_cold(S, f3(p.x + 0.0f, p.y + e, p.z + 0.0f), set1) -
                         scene_sdf_cold(S, f3(p.x - 0.0f, p.y - e, p.z - 0.0f), set1);
        const float nz = scene_sdf_cold(S, f3(p.x + 0.0f, p.y + 0.0f, p.z + e), set1) -
                         scene_sdf_cold(S, f3(p.x - 0.0f, p.y - 0.0f, p.z - e), set1);
        h.normal = normalize3(f3(nx, ny, nz));
        h.materialID = scene_sdf_material_hit(S, p, set1, hit_sel);
        h.lightID = -1.0f;
        return true;
    }
    return false;
}

// The analytic part of Intersection (SC:862-923) and of the object loop of
// LightSourceVisibilityCheck (SC:1121-1201): objectID = index of the last
// object whose test hit, -1 for none.
template <int FEAT = PT_FEAT_ALL>
PT_DI void intersect_analytic(const KScene& S, float3 org, float3 dir, Hit& h, int& objectID) {
    int id = -1;
    const int n0 = S.meta.n[0], n1 = S.meta.n[1], n2 = S.meta.n[2], n3 = S.meta.n[3], n4 = S.meta.n[4];
    int gi = 0;
#pragma unroll 1
    for (int i = 0; i < n0; i++, gi++) {
        const int b = 6 * i;
        const float3 pos = f3(S.objects[b], S.objects[b + 1], S.objects[b + 2]);
        if (sphere_intersect(org, dir, pos, S.objects[b + 3], (float)((int)S.objects[b + 4] - 1),
                             (float)((int)S.objects[b + 5] - 1), h))
            id = gi;
    }
#pragma unroll 1
    for (int i = 0; i < n1; i++, gi++) {
        const int b = S.meta.offset[1] + 5 * i;
        const float3 pos = f3(S.objects[b], S.objects[b + 1], S.objects[b + 2]);
        if (plane_intersect(org, dir, pos, (float)((int)S.objects[b + 3] - 1), (float)((int)S.objects[b + 4] - 1),
                            h))
            id = gi;
    }
    if constexpr ((FEAT & PT_FEAT_BOX) != 0) {
#pragma unroll 1
        for (int i = 0; i < n2; i++, gi++) {
            const int b = S.meta.offset[2] + 11 * i;
            const float3 pos = f3(S.objects[b], S.objects[b + 1], S.objects[b + 2]);
            const float3 size = f3(S.objects[b + 6], S.objects[b + 7], S.objects[b + 8]);
            if (!bounding_sphere(org, dir, pos, 0.25f * dot3(size, size))) continue;
            if (box_intersect(org, dir, pos, size, s_rotation(S, gi), (float)((int)S.objects[b + 9] - 1),
                              (float)((int)S.objects[b + 10] - 1), h))
                id = gi;
        }
    }
    if constexpr ((FEAT & PT_FEAT_LENS) != 0) {
#pragma unroll 1
        for (int i = 0; i < n3; i++, gi++) {
            const int b = S.meta.offset[3] + 12 * i;
            LensGeom L;
            L.pos = f3(S.objects[b], S.objects[b + 1], S.objects[b + 2]);
            L.radius = S.objects[b + 6];
            L.focal = S.objects[b + 7];
            L.thickness = S.objects[b + 8];
            L.converging = S.objects[b + 9] != 0.0f;
            if (!bounding_sphere(org, dir, L.pos, lens_bounding_radius2(L.radius, L.focal, L.thickness, L.converging)))
                continue;
            L.rot = s_rotation(S, gi);
            int isOutside = 1;
            if (lens_intersect(org, dir, L, (float)((int)S.objects[b + 10] - 1), (float)((int)S.objects[b + 11] - 1),
                               h, isOutside))
                id = gi;
        }
    }
    if constexpr ((FEAT & PT_FEAT_CYCLIDE) != 0) {
#pragma unroll 1
        for (int i = 0; i < n4; i++, gi++) {
            const int b = S.meta.offset[4] + 16 * i;
            const float3 pos = f3(S.objects[b], S.objects[b + 1], S.objects[b + 2]);
            if (!bounding_sphere(org, dir, pos, S.objects[b + 13])) continue;
            if (cyclide_intersect(S, org, dir, b, s_rotation(S, gi), h)) id = gi;
        }
    }
    objectID = id;
}

// Intersection (SC:862-934) / LightSourceVisibilityCheck's loop: the analytic
// objects, then sphere tracing of the SDFs (objectID -2 for an SDF hit).
template <int FEAT = PT_FEAT_ALL>
PT_DI void intersect_all(const KScene& S, float3 org, float3 dir, Hit& h, int& objectID) {
    intersect_analytic<FEAT>(S, org, dir, h, objectID);
    if constexpr ((FEAT & PT_FEAT_SDF) != 0) {
        if (S.meta.n[5] > 0) {
            if (sphere_trace(S, org, dir, h)) objectID = -2;
        }
    }
}
