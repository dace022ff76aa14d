// pt_geometry.cuh — analytic primitives, SDF plug-ins and sphere tracing.
//
// Each function restates the cited lines of src/shader.comp (SC) with the
// same operation order; the differences are GPU-side only: rotation matrices
// come from the per-upload table (KScene::rot) and objects are read straight
// from the launch's constant bank instead of being unpacked into structs.
// The functions are templates over the scalar type R (see pt_vec.cuh): the
// float instantiation is the shader's arithmetic, the double one the FP64
// reference renderer's; the scene data (KScene) is float in both.
#pragma once

#include "pt_features.h"
#include "pt_scene.cuh"

#define PT_PI 3.141592653589792623810034526344f  // SC:9
#define PT_ONEBYTHREE 0.3333333f                 // SC:10
#define PT_MAXDIST 1e5f                          // SC:8
// The same constants in precision R.
#define PT_PI_R(R) PT_LIT(R, 3.141592653589792623810034526344)
#define PT_ONEBYTHREE_R(R) PT_LIT(R, 0.3333333)

// A parameter type that takes no part in template argument deduction.
template <typename T> struct PtIdentity { using type = T; };
template <typename T> using ND = typename PtIdentity<T>::type;

template <typename R> struct HitT {
    R hitdist;
    V3<R> normal;
    R materialID;
    R lightID;
};
using Hit = HitT<float>;

// BoundingSphere, SC:263-276.
template <typename V> PT_DI bool bounding_sphere(V org, V dir, V pos, ND<SOf<V>> radius2) {
    using R = SOf<V>;
    const V lo = org - pos;
    const R b = dot3(dir, lo);
    const R c = dot3(lo, lo) - radius2;
    if ((b * b) < c) return false;
    if ((b >= R(0)) && (c >= R(0))) return false;
    return true;
}

// SphereIntersection, SC:289-317.
template <typename R>
PT_DI bool sphere_intersect(V3<R> org, V3<R> dir, V3<R> pos, ND<R> radius, ND<R> mat, ND<R> light, HitT<R>& h) {
    const V3<R> lo = org - pos;
    const R b = R(2) * dot3(dir, lo);
    const R c = dot3(lo, lo) - (radius * radius);
    const R disc = b * b - R(4) * c;
    if (disc < R(0)) return false;
    const R sqrtD = m_sqrt(disc);
    const R t1 = (-b - sqrtD) * R(0.5);
    const R t2 = (-b + sqrtD) * R(0.5);
    const R t = (t1 > R(0)) ? t1 : t2;
    const R isOutside = (t1 > R(0)) ? R(1) : R(-1);
    if (t < PT_LIT(R, 1e-4)) return false;
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
template <typename R>
PT_DI bool plane_intersect(V3<R> org, V3<R> dir, V3<R> pos, ND<R> mat, ND<R> light, HitT<R>& h) {
    const V3<R> lo = org - pos;
    const R t = -lo.y / dir.y;
    if (t < PT_LIT(R, 1e-4)) return false;
    if (t < h.hitdist) {
        h.hitdist = t;
        const R d = R(0) * dir.x + R(1) * dir.y + R(0) * dir.z;  // faceforward: dot(Nref, I)
        h.normal = (d < R(0)) ? v3<R>(R(0), R(1), R(0)) : v3<R>(R(-0.0), R(-1), R(-0.0));
        h.materialID = mat;
        h.lightID = light;
        return true;
    }
    return false;
}

// BoxIntersection, SC:337-364 (matrix from KScene::rot).
template <typename R>
PT_DI bool box_intersect(V3<R> org, V3<R> dir_w, V3<R> pos, V3<R> size, const M3<R>& m, ND<R> mat, ND<R> light,
                         HitT<R>& h) {
    const V3<R> lo = mul_vm(org - pos, m);
    const V3<R> dir = mul_vm(dir_w, m);
    const V3<R> invdir = v3<R>(R(1) / dir.x, R(1) / dir.y, R(1) / dir.z);
    const V3<R> tMin0 = fma3(size, v3<R>(R(-0.5), R(-0.5), R(-0.5)), -lo) * invdir;
    const V3<R> tMax0 = fma3(size, v3<R>(R(0.5), R(0.5), R(0.5)), -lo) * invdir;
    const V3<R> a = min3(tMin0, tMax0), bb = max3(tMin0, tMax0);
    const R t1 = m_fmax(m_fmax(a.x, a.y), a.z);
    const R t2 = m_fmin(m_fmin(bb.x, bb.y), bb.z);
    const R t = (t1 < R(0)) ? t2 : t1;
    if ((t1 > t2) || (t < PT_LIT(R, 1e-4))) return false;
    if (t < h.hitdist) {
        h.hitdist = t;
        const V3<R> p = abs3((lo + dir * t) / size);
        const R mx = m_fmax(m_fmax(p.x, p.y), p.z);
        const V3<R> st = v3<R>(step_glsl(mx, p.x), step_glsl(mx, p.y), step_glsl(mx, p.z));
        const V3<R> sg = v3<R>(-sign_glsl(dir.x), -sign_glsl(dir.y), -sign_glsl(dir.z));
        h.normal = mul_mv(m, st * sg);
        h.materialID = mat;
        h.lightID = light;
        return true;
    }
    return false;
}

// Lens geometry shared by the camera lens and scene lenses.
template <typename R> struct LensGeomT {
    V3<R> pos;
    M3<R> rot;
    R radius;        // lens aperture radius
    R focal;         // focal length
    R thickness;
    bool converging;
};
using LensGeom = LensGeomT<float>;

// SphereSliceIntersection, SC:366-417.
template <typename R>
PT_DI bool slice_intersect(V3<R> org_w, V3<R> dir_w, const LensGeomT<R>& L, ND<R> sliceRadius, ND<R> sliceSize,
                           bool is1st, ND<R> localSlicePos, bool isSideInvert, ND<R> mat, ND<R> light, HitT<R>& h,
                           int& isOutside) {
    const R sliceOffset = sliceRadius - sliceSize;
    V3<R> org = mul_vm(org_w - L.pos, L.rot);
    if (is1st) {
        org.x += localSlicePos - sliceSize - sliceOffset;
    } else {
        org.x -= localSlicePos - sliceSize - sliceOffset;
    }
    const V3<R> dir = mul_vm(dir_w, L.rot);
    const R b = R(2) * dot3(dir, org);
    const R c = dot3(org, org) - (sliceRadius * sliceRadius);
    const R disc = b * b - R(4) * c;
    R t = R(1e6);
    int isOut = 1;
    if (disc < R(0)) return false;
    const R sqrtD = m_sqrt(disc);
    R t1 = (-b - sqrtD) * R(0.5);
    R t2 = (-b + sqrtD) * R(0.5);
    if (is1st) {
        t1 = (m_fma(dir.x, t1, org.x) > -sliceOffset) ? R(1e6) : t1;
        t2 = (m_fma(dir.x, t2, org.x) > -sliceOffset) ? R(1e6) : t2;
    } else {
        t1 = (m_fma(dir.x, t1, org.x) < sliceOffset) ? R(1e6) : t1;
        t2 = (m_fma(dir.x, t2, org.x) < sliceOffset) ? R(1e6) : t2;
    }
    t = (t1 > R(0)) ? t1 : t;
    if (t2 < t) {
        t = t2;
        isOut = -1;
    }
    if (t < PT_LIT(R, 1e-4)) return false;
    if (t < h.hitdist) {
        h.hitdist = t;
        h.normal = mul_mv(L.rot, normalize3(fma3s(dir, t, org) * (R)isOut));
        isOutside = (!isSideInvert) ? isOut : -isOut;
        h.materialID = mat;
        h.lightID = light;
        return true;
    }
    return false;
}

// LensIntersection, SC:419-448.
template <typename R>
PT_DI bool lens_intersect(V3<R> org, V3<R> dir, const LensGeomT<R>& L, ND<R> mat, ND<R> light, HitT<R>& h,
                          int& isOutside) {
    const R lensThicknessHalf = R(2) * L.focal - m_sqrt(R(4) * L.focal * L.focal - L.radius * L.radius);
    R lensSlicePos = R(0.5) * (L.converging ? L.thickness : -L.thickness);
    if (L.converging) lensSlicePos += lensThicknessHalf;
    const R sliceRadius = R(2) * L.focal;
    bool hit = false;
#pragma unroll
    for (int i = 0; i < 2; i++) {
        if (slice_intersect(org, dir, L, sliceRadius, lensThicknessHalf, i == 0, lensSlicePos, !L.converging, mat,
                            light, h, isOutside))
            hit = true;
    }
    return hit;
}

template <typename R> PT_DI R lens_bounding_radius2(R radius, R focal, R thickness, bool converging) {
    R br;
    if (converging) {
        br = (radius * radius) + (R(0.25) * thickness * thickness);
    } else {
        br = R(0.5) * thickness + R(2) * focal - m_sqrt(R(4) * focal * focal - radius * radius);
        br = br * br + radius * radius;
    }
    return br;
}

// ---------------------------------------------------------------------------
// Quartic / cubic solvers (SC:450-541) and the Dupin cyclide (SC:633-679).
template <typename R> PT_DI R eval_quadratic(ND<R> a, ND<R> b, ND<R> c, R x) { return x * (x * a + b) + c; }
template <typename R> PT_DI R eval_cubic(ND<R> a, ND<R> b, ND<R> c, ND<R> d, R x) { return x * (x * (x * a + b) + c) + d; }
template <typename R> PT_DI R eval_quartic(ND<R> a, ND<R> b, ND<R> c, ND<R> d, ND<R> e, R x) {
    return x * (x * (x * (x * a + b) + c) + d) + e;
}

// SolveCubic, SC:474-503; only the first root is consumed by SolveQuartic.
template <typename R> PT_DI R solve_cubic_first(R b, R c, R d) {
    const R bdiv3 = b * PT_ONEBYTHREE_R(R);
    const R Q = c * PT_ONEBYTHREE_R(R) - bdiv3 * bdiv3;
    const R Rr = PT_LIT(R, 0.5) * bdiv3 * c - bdiv3 * bdiv3 * bdiv3 - PT_LIT(R, 0.5) * d;
    const R D = Q * Q * Q + Rr * Rr;
    R x;
    if (D > PT_LIT(R, 0.0)) {
        const R u = Rr + m_sqrt(D);
        const R v = Rr - m_sqrt(D);
        const R S = sign_glsl(u) * m_pow(m_fabs(u), PT_ONEBYTHREE_R(R));
        const R T = sign_glsl(v) * m_pow(m_fabs(v), PT_ONEBYTHREE_R(R));
        x = S + T - bdiv3;
    } else {
        const R sqrtnegQ = m_sqrt(-Q);
        const R thetadiv3 = m_acos(Rr / (sqrtnegQ * sqrtnegQ * sqrtnegQ)) * PT_ONEBYTHREE_R(R);
        x = PT_LIT(R, 2.0) * sqrtnegQ * m_cos(thetadiv3) - bdiv3;
    }
#pragma unroll
    for (int i = 0; i < 2; i++) x -= eval_cubic(PT_LIT(R, 1.0), b, c, d, x) / eval_quadratic(PT_LIT(R, 3.0), PT_LIT(R, 2.0) * b, c, x);
    return x;
}

// SolveQuartic, SC:505-541, folded into "smallest positive real root below t".
template <typename R> PT_DI R solve_quartic_min_positive(R a, R b, R c, R d, R e) {
    const R inva = PT_LIT(R, 1.0) / a;
    const R inva2 = inva * PT_LIT(R, 0.5);
    const R inva2a2 = inva2 * inva2;
    const R bb = b * b;
    const R p = -PT_LIT(R, 1.5) * bb * inva2a2 + c * inva;
    const R q = bb * b * inva2a2 * inva2 - b * c * inva * inva2 + d * inva;
    const R r = -PT_LIT(R, 0.1875) * bb * bb * inva2a2 * inva2a2 + PT_LIT(R, 0.5) * c * bb * inva2a2 * inva2 - b * d * inva2a2 + e * inva;
    const R sx = solve_cubic_first(PT_LIT(R, 0.5) * -p, -r, PT_LIT(R, 0.5) * p * r - PT_LIT(R, 0.125) * q * q);
    R t = PT_LIT(R, 1e6);
    const R s2subp = PT_LIT(R, 2.0) * sx - p;
    if (s2subp < PT_LIT(R, 0.0)) return t;
    const R invs2subp = -PT_LIT(R, 2.0) * sx - p;
    const R sqrts2subp = m_sqrt(s2subp);
    const R q2divsqrt = PT_LIT(R, 2.0) * q / sqrts2subp;
    const R invaddq2div = invs2subp + q2divsqrt;
    const R invsubq2div = invs2subp - q2divsqrt;
    const R bdiv4a = PT_LIT(R, 0.25) * inva * b;
    R r0 = PT_LIT(R, 0.0), r1 = PT_LIT(R, 0.0), r2 = PT_LIT(R, 0.0), r3 = PT_LIT(R, 0.0);
    const bool re01 = invaddq2div >= PT_LIT(R, 0.0);
    const bool re23 = invsubq2div >= PT_LIT(R, 0.0);
    if (re01) {
        const R sq = m_sqrt(invaddq2div);
        r0 = PT_LIT(R, 0.5) * (-sqrts2subp + PT_LIT(R, 1.0) * sq) - bdiv4a;
        r1 = PT_LIT(R, 0.5) * (-sqrts2subp + -PT_LIT(R, 1.0) * sq) - bdiv4a;
        r0 -= eval_quartic(a, b, c, d, e, r0) / eval_cubic(PT_LIT(R, 4.0) * a, PT_LIT(R, 3.0) * b, PT_LIT(R, 2.0) * c, d, r0);
        r1 -= eval_quartic(a, b, c, d, e, r1) / eval_cubic(PT_LIT(R, 4.0) * a, PT_LIT(R, 3.0) * b, PT_LIT(R, 2.0) * c, d, r1);
    }
    if (re23) {
        const R sq = m_sqrt(invsubq2div);
        r2 = PT_LIT(R, 0.5) * (sqrts2subp + PT_LIT(R, 1.0) * sq) - bdiv4a;
        r3 = PT_LIT(R, 0.5) * (sqrts2subp + -PT_LIT(R, 1.0) * sq) - bdiv4a;
        r2 -= eval_quartic(a, b, c, d, e, r2) / eval_cubic(PT_LIT(R, 4.0) * a, PT_LIT(R, 3.0) * b, PT_LIT(R, 2.0) * c, d, r2);
        r3 -= eval_quartic(a, b, c, d, e, r3) / eval_cubic(PT_LIT(R, 4.0) * a, PT_LIT(R, 3.0) * b, PT_LIT(R, 2.0) * c, d, r3);
    }
    // DupinCyclide SC:648-655: scan the real roots in order.
    if (re01) {
        if ((r0 < t) && (r0 > PT_LIT(R, 0.0))) t = r0;
        if ((r1 < t) && (r1 > PT_LIT(R, 0.0))) t = r1;
    }
    if (re23) {
        if ((r2 < t) && (r2 > PT_LIT(R, 0.0))) t = r2;
        if ((r3 < t) && (r3 > PT_LIT(R, 0.0))) t = r3;
    }
    return t;
}

template <typename V> PT_DI V sw_xzy(V v) { return V{v.x, v.z, v.y}; }
template <typename V> PT_DI V sw_yzx(V v) { return V{v.y, v.z, v.x}; }
template <typename V> PT_DI V sw_zxy(V v) { return V{v.z, v.x, v.y}; }

// DupinCyclide, SC:633-679.  base = R offset of the cyclide in objects[].
template <typename R>
PT_DI bool cyclide_intersect(const KScene& S, V3<R> org, V3<R> dir, int base, const M3<R>& m, HitT<R>& h) {
    const V3<R> pos = v3<R>(S.objects[base], S.objects[base + 1], S.objects[base + 2]);
    const V3<R> scale = v3<R>(S.objects[base + 6], S.objects[base + 7], S.objects[base + 8]);
    const R A = S.objects[base + 9], B = S.objects[base + 10];
    const R C = S.objects[base + 11], Dd = S.objects[base + 12];
    const V3<R> o = sw_xzy(mul_vm(org - pos, m) / scale);
    const V3<R> d = sw_xzy(mul_vm(dir, m) / scale);
    const V3<R> dd = d * d, oo = o * o, od = o * d;
    const V3<R> dyzx = sw_yzx(d), dzxy = sw_zxy(d), oyzx = sw_yzx(o), ozxy = sw_zxy(o);
    const R a4 = dot3(dd, dd) + PT_LIT(R, 2.0) * dot3(dd, dyzx * dyzx);
    const R a3 = PT_LIT(R, 4.0) * (dot3(o, dd * d) + dot3(od, dyzx * dyzx) + dot3(od, dzxy * dzxy));
    const R a2 = PT_LIT(R, 6.0) * dot3(oo, dd) + PT_LIT(R, 8.0) * dot3(od, oyzx * dyzx) +
                     PT_LIT(R, 2.0) * (dot3(oo, dyzx * dyzx) + dot3(oo, dzxy * dzxy)) + PT_LIT(R, 2.0) * (B * B - Dd * Dd) * dot3(d, d) -
                     PT_LIT(R, 4.0) * (A * A * d.x * d.x + B * B * d.y * d.y);
    const R a1 = PT_LIT(R, 4.0) * (dot3(oo * o, d) + dot3(oo, oyzx * dyzx) + dot3(oo, ozxy * dzxy) + PT_LIT(R, 2.0) * A * C * Dd * d.x +
                             (B * B - Dd * Dd) * dot3(o, d) - PT_LIT(R, 2.0) * (A * A * o.x * d.x + B * B * o.y * d.y));
    const R a0 = dot3(oo, oo) + PT_LIT(R, 2.0) * dot3(oo, oyzx * oyzx) + B * B * B * B + Dd * Dd * Dd * Dd -
                     PT_LIT(R, 2.0) * B * B * Dd * Dd - PT_LIT(R, 4.0) * C * C * Dd * Dd + PT_LIT(R, 8.0) * A * C * Dd * o.x +
                     PT_LIT(R, 2.0) * (B * B - Dd * Dd) * dot3(o, o) - PT_LIT(R, 4.0) * (A * A * o.x * o.x + B * B * o.y * o.y);
    const R t = solve_quartic_min_positive(a4, a3, a2, a1, a0);
    if (t < h.hitdist) {
        h.hitdist = t;
        const R x = o.x + d.x * t;
        const R y = o.y + d.y * t;
        const R z = o.z + d.z * t;
        const R term1 = x * x + y * y + z * z + B * B - Dd * Dd;
        const V3<R> n = v3<R>(PT_LIT(R, 4.0) * (x * term1 - PT_LIT(R, 2.0) * A * (A * x - C * Dd)), PT_LIT(R, 4.0) * z * term1,
                            PT_LIT(R, 4.0) * y * (term1 - PT_LIT(R, 2.0) * B * B));
        h.normal = normalize3(n);
        h.materialID = (R)((int)S.objects[base + 14] - 1);
        h.lightID = (R)((int)S.objects[base + 15] - 1);
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
template <typename R> PT_DI bool thritorius_intersect(V3<R> org, V3<R> dir, HitT<R>& h) {
    if (!bounding_sphere(org, dir, v3<R>(PT_LIT(R, 0.0), PT_LIT(R, 0.0), PT_LIT(R, 0.0)), PT_LIT(R, 4.05))) return false;
    const V3<R> o = sw_xzy(org), d = sw_xzy(dir);
    const V3<R> ddd = (d * d) * d;
    const V3<R> d10 = v3<R>(d.x, d.y, PT_LIT(R, 10.0) * d.z), o10 = v3<R>(o.x, o.y, PT_LIT(R, 10.0) * o.z);
    const R a4 = dot3(d10, ddd) + PT_LIT(R, 2.0) * dot3(d * d, sw_yzx(d) * sw_yzx(d));
    const V3<R> dd2 = v3<R>(d.y * d.y + d.z * d.z, d.x * d.x + d.z * d.z, d.x * d.x + d.y * d.y);
    const R a3 = PT_LIT(R, 4.0) * (dot3(o10, ddd) + dot3(o * d, dd2)) + PT_LIT(R, 2.0) * d.y * d.y * d.y - PT_LIT(R, 6.0) * d.x * d.x * d.y;
    const V3<R> oxxy = v3<R>(o.x, o.x, o.y), dxxy = v3<R>(d.x, d.x, d.y), oyzz = v3<R>(o.y, o.z, o.z), dyzz = v3<R>(d.y, d.z, d.z);
    const R a2 = PT_LIT(R, 6.0) * dot3(o10, (o * d) * d) +
                     PT_LIT(R, 2.0) * ((o.x * o.x * (d.y * d.y) + o.y * o.y * (d.x * d.x)) +
                             (o.x * o.x * (d.z * d.z) + o.z * o.z * (d.x * d.x)) +
                             (o.y * o.y * (d.z * d.z) + o.z * o.z * (d.y * d.y))) +
                     PT_LIT(R, 8.0) * dot3(oxxy * dxxy, oyzz * dyzz) + PT_LIT(R, 6.0) * o.y * d.y * d.y - PT_LIT(R, 6.0) * o.y * d.x * d.x -
                     PT_LIT(R, 12.0) * o.x * d.x * d.y - PT_LIT(R, 12.0) * d.z * d.z;
    const R a1 = PT_LIT(R, 4.0) * (dot3((o10 * o) * o, d) + (o.x * o.x * (o.y * d.y) + o.x * o.x * (o.z * d.z)) +
                             (o.y * o.y * (o.x * d.x) + o.y * o.y * (o.z * d.z)) +
                             (o.z * o.z * (o.x * d.x) + o.z * o.z * (o.y * d.y))) +
                     PT_LIT(R, 6.0) * o.y * o.y * d.y - PT_LIT(R, 6.0) * o.x * o.x * d.y - PT_LIT(R, 12.0) * o.x * o.y * d.x - PT_LIT(R, 24.0) * o.z * d.z;
    const R a0 = dot3(o10, (o * o) * o) + PT_LIT(R, 2.0) * dot3(oxxy * oxxy, oyzz * oyzz) + PT_LIT(R, 2.0) * o.y * o.y * o.y -
                     PT_LIT(R, 6.0) * o.x * o.x * o.y - PT_LIT(R, 12.0) * o.z * o.z + PT_LIT(R, 1.0);
    const R t = solve_quartic_min_positive(a4, a3, a2, a1, a0);
    if (t < h.hitdist) {
        h.hitdist = t;
        const R x = o.x + d.x * t;
        const R y = o.y + d.y * t;
        const R z = o.z + d.z * t;
        V3<R> n = v3<R>(PT_LIT(R, 4.0) * x * x * x + PT_LIT(R, 4.0) * x * y * y - PT_LIT(R, 12.0) * x * y + PT_LIT(R, 4.0) * x * z * z,
                      PT_LIT(R, 40.0) * z * z * z + PT_LIT(R, 4.0) * x * x * z + PT_LIT(R, 4.0) * y * y * z - PT_LIT(R, 24.0) * z,
                      PT_LIT(R, 4.0) * y * y * y + PT_LIT(R, 4.0) * x * x * y - PT_LIT(R, 6.0) * x * x + PT_LIT(R, 6.0) * y * y + PT_LIT(R, 4.0) * y * z * z);
        if ((o.x * o.x * (o.x * o.x + PT_LIT(R, 2.0) * o.y * o.y - PT_LIT(R, 6.0) * o.y + PT_LIT(R, 2.0) * o.z * o.z) +
             o.y * o.y * (o.y * o.y + PT_LIT(R, 2.0) * o.y + PT_LIT(R, 2.0) * o.z * o.z) + o.z * o.z * (PT_LIT(R, 10.0) * o.z * o.z - PT_LIT(R, 12.0)) +
             PT_LIT(R, 1.0)) < PT_LIT(R, 0.0))
            n = n * -PT_LIT(R, 1.0);
        h.normal = normalize3(n);
        h.materialID = PT_LIT(R, 1.0);
        h.lightID = -PT_LIT(R, 1.0);
        return true;
    }
    return false;
}

// SmoothCuboid, SC:590-631: x^4 + y^4 + z^4 = 1 at the origin.
template <typename R> PT_DI bool smooth_cuboid_intersect(V3<R> o, V3<R> d, HitT<R>& h) {
    if (!bounding_sphere(o, d, v3<R>(PT_LIT(R, 0.0), PT_LIT(R, 0.0), PT_LIT(R, 0.0)), PT_LIT(R, 1.80))) return false;
    const R a4 = dot3(d * d, d * d);
    const R a3 = PT_LIT(R, 4.0) * dot3(o, (d * d) * d);
    const R a2 = PT_LIT(R, 6.0) * dot3(o * o, d * d);
    const R a1 = PT_LIT(R, 4.0) * dot3((o * o) * o, d);
    const R a0 = dot3(o * o, o * o) - PT_LIT(R, 1.0);
    const R t = solve_quartic_min_positive(a4, a3, a2, a1, a0);
    if (t < h.hitdist) {
        h.hitdist = t;
        V3<R> n = fma3s(d, t, o);
        n = (n * n) * n;
        if (dot3(o * o, o * o) < PT_LIT(R, 1.0)) n = n * -PT_LIT(R, 1.0);
        h.normal = normalize3(n);
        h.materialID = PT_LIT(R, 3.0);
        h.lightID = -PT_LIT(R, 1.0);
        return true;
    }
    return false;
}

// ---------------------------------------------------------------------------
// SDF plug-ins: the four snippets of sdfs/<name>.glsl as __device__ functions
// with the snippets' signature `R sdf(vec3 p)` / `R sdfmaterial(vec3 p)`.

// smin, SC:686-702.
template <typename R> PT_DI R smin1(R x, R y) {
    R k = PT_LIT(R, 0.02);
    k *= PT_LIT(R, 6.0);
    const R h = m_fmax(k - m_fabs(x - y), PT_LIT(R, 0.0)) / k;
    const R m = h * h * h * PT_LIT(R, 0.5);
    const R s = m * k * PT_ONEBYTHREE_R(R);
    return m_fmin(x, y) - s;
}
template <typename V, typename R = SOf<V>> PT_DI V smin2(V x, V y) {
    R k = PT_LIT(R, 0.02);
    k *= PT_LIT(R, 6.0);
    const R h = m_fmax(k - m_fabs(x.x - y.x), PT_LIT(R, 0.0)) / k;
    const R m = h * h * h * PT_LIT(R, 0.5);
    const R s = m * k * PT_ONEBYTHREE_R(R);
    return (x.x < y.x) ? v2<R>(x.x - s, x.y + (y.y - x.y) * m)
                       : v2<R>(y.x - s, x.y + (y.y - x.y) * (PT_LIT(R, 1.0) - m));
}

namespace sdf_blob {  // sdfs/blob.glsl
template <typename V, typename R = SOf<V>> PT_DI R sdf(V p) {
    const R s1 = length3(p) - PT_LIT(R, 1.0);
    const R s2 = length3(v3<R>(p.x, p.y - PT_LIT(R, 1.0), p.z)) - PT_LIT(R, 0.7);
    const R s3 = length3(v3<R>(p.x - PT_LIT(R, 0.25), p.y - PT_LIT(R, 1.25), p.z - PT_LIT(R, 0.5))) - PT_LIT(R, 0.25);
    const R s4 = length3(v3<R>(p.x + PT_LIT(R, 0.25), p.y - PT_LIT(R, 1.25), p.z - PT_LIT(R, 0.5))) - PT_LIT(R, 0.25);
    return smin1(smin1(smin1(s1, s2), s3), s4);
}
template <typename V, typename R = SOf<V>> PT_DI R sdfmaterial(V p, const float* m) {
    const V2<R> s1 = v2<R>(length3(p) - PT_LIT(R, 1.0), m[0]);
    const V2<R> s2 = v2<R>(length3(v3<R>(p.x, p.y - PT_LIT(R, 1.0), p.z)) - PT_LIT(R, 0.7), m[1]);
    const V2<R> s3 = v2<R>(length3(v3<R>(p.x - PT_LIT(R, 0.25), p.y - PT_LIT(R, 1.25), p.z - PT_LIT(R, 0.5))) - PT_LIT(R, 0.25), m[2]);
    const V2<R> s4 = v2<R>(length3(v3<R>(p.x + PT_LIT(R, 0.25), p.y - PT_LIT(R, 1.25), p.z - PT_LIT(R, 0.5))) - PT_LIT(R, 0.25), m[2]);
    return smin2(smin2(smin2(s1, s2), s3), s4).y;
}
}  // namespace sdf_blob

namespace sdf_mandelbulb {  // sdfs/mandelbulb.glsl (power 8, 4 iterations, bailout 16)
template <typename V, typename R = SOf<V>> PT_DI R sdf(V p) {
    V3<R> z = p;
    R r = length3(z);
    R dr = PT_LIT(R, 1.0);
#pragma unroll 1
    for (int i = 0; i < 4; i++) {
        dr = PT_LIT(R, 8.0) * pow_pos_int<7>(r) * dr + PT_LIT(R, 1.0);  // r = length(z): +0, positive, +inf or NaN
        const R invr = PT_LIT(R, 1.0) / r;
        const R invl = PT_LIT(R, 1.0) / m_sqrt(z.x * z.x + z.z * z.z);
        r *= r;
        r *= r;
        r *= r;
        const R cost = z.z * invl;
        const R cosp = z.y * invr;
        const R sint = z.x * invl;
        const R sinp = invr / invl;
        const R cost2 = cost * cost;
        const R cosp2 = cosp * cosp;
        const R cost8 =
            m_fma(m_fma(m_fma(m_fma(PT_LIT(R, 128.0), cost2, -PT_LIT(R, 256.0)), cost2, PT_LIT(R, 160.0)), cost2, -PT_LIT(R, 32.0)), cost2, PT_LIT(R, 1.0));
        const R cosp8 =
            m_fma(m_fma(m_fma(m_fma(PT_LIT(R, 128.0), cosp2, -PT_LIT(R, 256.0)), cosp2, PT_LIT(R, 160.0)), cosp2, -PT_LIT(R, 32.0)), cosp2, PT_LIT(R, 1.0));
        const R sint8 = m_fma(m_fma(m_fma(PT_LIT(R, 128.0), cost2, -PT_LIT(R, 192.0)), cost2, PT_LIT(R, 80.0)), cost2, -PT_LIT(R, 8.0)) * sint * cost;
        const R sinp8 = m_fma(m_fma(m_fma(PT_LIT(R, 128.0), cosp2, -PT_LIT(R, 192.0)), cosp2, PT_LIT(R, 80.0)), cosp2, -PT_LIT(R, 8.0)) * sinp * cosp;
        z = v3<R>(sint8 * sinp8, cosp8, cost8 * sinp8) * r;
        z = z + p;
        r = length3(z);
        if (r > PT_LIT(R, 16.0)) break;
    }
    return PT_LIT(R, 0.5) * m_log_inline(r) * r / dr;  // inlined: the march loop's hottest call
}
template <typename V, typename R = SOf<V>> PT_DI R sdfmaterial(V p, const float* m) {
    const R factor = dot3(p, p);
    return mix_glsl<R>(m[0], m[1], factor / (PT_LIT(R, 0.8) + factor));
}
}  // namespace sdf_mandelbulb

namespace sdf_menger {  // sdfs/menger.glsl
template <typename V, typename R = SOf<V>> PT_DI R sdf(V p) {
    const V3<R> q = abs3(p) - v3<R>(PT_LIT(R, 1.0), PT_LIT(R, 1.0), PT_LIT(R, 1.0));
    R d = length3(max3(q, v3<R>(PT_LIT(R, 0.0), PT_LIT(R, 0.0), PT_LIT(R, 0.0)))) + m_fmin(m_fmax(q.x, m_fmax(q.y, q.z)), PT_LIT(R, 0.0));
    R s = PT_LIT(R, 1.0);
#pragma unroll 1
    for (int m = 0; m < 5; m++) {
        const V3<R> ps = p * s;
        const V3<R> a = v3<R>(mod_glsl(ps.x, PT_LIT(R, 2.0)) - PT_LIT(R, 1.0), mod_glsl(ps.y, PT_LIT(R, 2.0)) - PT_LIT(R, 1.0), mod_glsl(ps.z, PT_LIT(R, 2.0)) - PT_LIT(R, 1.0));
        s *= PT_LIT(R, 3.0);
        const V3<R> r =
            v3<R>(m_fabs(PT_LIT(R, 1.0) - PT_LIT(R, 3.0) * m_fabs(a.x)), m_fabs(PT_LIT(R, 1.0) - PT_LIT(R, 3.0) * m_fabs(a.y)), m_fabs(PT_LIT(R, 1.0) - PT_LIT(R, 3.0) * m_fabs(a.z)));
        const R da = m_fmax(r.x, r.y);
        const R db = m_fmax(r.y, r.z);
        const R dc = m_fmax(r.z, r.x);
        const R c = (m_fmin(da, m_fmin(db, dc)) - PT_LIT(R, 1.0)) / s;
        d = m_fmax(d, c);
    }
    return d;
}
}  // namespace sdf_menger

namespace sdf_terrain {  // sdfs/terrain.glsl
template <typename R> PT_DI R height(R x) {
    return m_sin_inline(PT_LIT(R, 0.0625) * x) + m_sin_inline(PT_LIT(R, 0.125) * (x + PT_LIT(R, 10.0))) + PT_LIT(R, 0.25) * m_sin_inline(PT_LIT(R, 0.25) * x) + PT_LIT(R, 0.125) * m_sin_inline(PT_LIT(R, 0.5) * x) +
           PT_LIT(R, 0.25) * m_sin_inline(x) + PT_LIT(R, 0.25) * m_sin_inline(PT_LIT(R, 2.0) * x + PT_LIT(R, 1.0)) + PT_LIT(R, 0.125) * m_sin_inline(PT_LIT(R, 4.0) * x + PT_LIT(R, 2.0)) +
           PT_LIT(R, 0.0625) * m_sin_inline(PT_LIT(R, 8.0) * x + PT_LIT(R, 1.0)) + PT_LIT(R, 0.03125) * m_sin_inline(PT_LIT(R, 16.0) * x + PT_LIT(R, 5.0)) + PT_LIT(R, 0.015625) * m_sin_inline(PT_LIT(R, 32.0) * x) +
           PT_LIT(R, 0.0078125) * m_sin_inline(PT_LIT(R, 64.0) * x);
}
template <typename V> PT_DI SOf<V> sdf(V p) { return p.y - (height(p.x) + height(p.z)); }
}  // namespace sdf_terrain

// A scene's SDF slot `slot` with plug-in `kind`.  PT_SDF_CUSTOM slots hold
// GLSL compiled at run time: the module built for them (pt_jit.cu) defines
// pt_user_sdf / pt_user_material (FP32 kernels) or pt_user_sdf_d /
// pt_user_material_d (the FP64 renderer) before including these headers;
// the precompiled kernels never see that kind.
//
// PT_SDF_KINDS (bit k: kind k) lists the kinds a kernel evaluates: a run-time
// compiled march kernel is given those of the scenes it renders, so the code
// of the other built-in SDFs is not in it; other kernels take every kind.
#ifndef PT_SDF_KINDS
#define PT_SDF_KINDS 0xFFFFFFFFu
#endif
static_assert(PT_SDF_BLOB == 1 && PT_SDF_MANDELBULB == 2 && PT_SDF_MENGER == 3 && PT_SDF_TERRAIN == 4,
              "the bit positions tested in plugin_sdf and plugin_material");
template <typename V, typename R = SOf<V>> PT_DI R plugin_sdf(int kind, int slot, V p) {
    switch (kind) {
#if (PT_SDF_KINDS >> 2) & 1u
        case PT_SDF_MANDELBULB: return sdf_mandelbulb::sdf(p);
#endif
#if (PT_SDF_KINDS >> 3) & 1u
        case PT_SDF_MENGER: return sdf_menger::sdf(p);
#endif
#if (PT_SDF_KINDS >> 1) & 1u
        case PT_SDF_BLOB: return sdf_blob::sdf(p);
#endif
#if (PT_SDF_KINDS >> 4) & 1u
        case PT_SDF_TERRAIN: return sdf_terrain::sdf(p);
#endif
#if defined(PT_JIT_USER_SDF)
        case PT_SDF_CUSTOM:
            if constexpr (sizeof(R) == 4) {
                return pt_user_sdf(slot, p);
            } else {
                return pt_user_sdf_d(slot, p);  // the FP64 renderer's module
            }
#endif
        default: return R(PT_MAXDIST);
    }
}
template <typename V, typename R = SOf<V>> PT_DI R plugin_material(const pt_sdf_plugin& pl, int slot, V p) {
    if (pl.material_mode == PT_SDFMAT_CONSTANT) return R(pl.material[0]);
    switch (pl.kind) {
#if (PT_SDF_KINDS >> 1) & 1u
        case PT_SDF_BLOB: return sdf_blob::sdfmaterial(p, pl.material);
#endif
#if (PT_SDF_KINDS >> 2) & 1u
        case PT_SDF_MANDELBULB: return sdf_mandelbulb::sdfmaterial(p, pl.material);
#endif
#if defined(PT_JIT_USER_SDF)
        case PT_SDF_CUSTOM:
            if constexpr (sizeof(R) == 4) {
                return pt_user_material(slot, p);
            } else {
                return pt_user_material_d(slot, p);
            }
#endif
        default: return R(pl.material[0]);
    }
}
template <typename R> PT_DI V3<R> sdf_pos(const KScene& S, int i) {
    return v3<R>(S.sdfs[6 * i], S.sdfs[6 * i + 1], S.sdfs[6 * i + 2]);
}

// SDF() with the lines InsertSDF splices in (src/pathtracer.cpp:2004-2054):
// in scene order, sdf = min(sdf, SDFi(p - pos_i)) for every bit i of set1.
template <typename V, typename R = SOf<V>> PT_DI R scene_sdf(const KScene& S, V p, uint32_t set1) {
    R sdf = R(PT_MAXDIST);
#if defined(PT_ONE_SDF)
    // A run-time compiled kernel for scenes whose one SDF is scene GLSL in
    // slot 0: the loop below with its one trip written out (same operations).
    if (set1 & 1u) sdf = m_fmin(sdf, plugin_sdf(PT_SDF_CUSTOM, S.meta.custom_base, p - sdf_pos<R>(S, 0)));
    return sdf;
#endif
    uint32_t bits = set1 & ((S.meta.nplug >= 32) ? 0xFFFFFFFFu : ((1u << S.meta.nplug) - 1u));
    while (bits) {
        const int i = __ffs(bits) - 1;
        bits &= bits - 1u;
        const int kind = S.plug[i].kind;
        if (kind != PT_SDF_NONE) sdf = m_fmin(sdf, plugin_sdf(kind, S.meta.custom_base + i, p - sdf_pos<R>(S, i)));
    }
    return sdf;
}
// scene_sdf that also reports the SDF whose material SDFMATERIAL() picks at
// p (SC:713-719: the last i with !(running minimum < d_i); -1 for none), so
// a march that converged at p needs only that SDF's material function there.
template <typename V, typename R = SOf<V>> PT_DI R scene_sdf_sel(const KScene& S, V p, uint32_t set1, int& sel) {
    R sdf = R(PT_MAXDIST);
    sel = -1;
#if defined(PT_ONE_SDF)
    if (set1 & 1u) {  // as in scene_sdf
        const R di = plugin_sdf(PT_SDF_CUSTOM, S.meta.custom_base, p - sdf_pos<R>(S, 0));
        if (!(sdf < di)) sel = 0;
        sdf = m_fmin(sdf, di);
    }
    return sdf;
#endif
    uint32_t bits = set1 & ((S.meta.nplug >= 32) ? 0xFFFFFFFFu : ((1u << S.meta.nplug) - 1u));
    while (bits) {
        const int i = __ffs(bits) - 1;
        bits &= bits - 1u;
        const int kind = S.plug[i].kind;
        if (kind != PT_SDF_NONE) {
            const R di = plugin_sdf(kind, S.meta.custom_base + i, p - sdf_pos<R>(S, i));
            if (!(sdf < di)) sel = i;
            sdf = m_fmin(sdf, di);
        }
    }
    return sdf;
}
// Out-of-line copy for the cold call sites (sign at the origin, normals).
template <typename V, typename R = SOf<V>>
static __device__ __noinline__ R scene_sdf_cold(const KScene& S, V p, uint32_t set1) { return scene_sdf(S, p, set1); }

// SDFMATERIAL() with the spliced minMaterial lines (SC:681-683, SC:713-719).
template <typename V, typename R = SOf<V>>
static __device__ __noinline__ R scene_sdf_material(const KScene& S, V p, uint32_t set1) {
    R sdf = R(PT_MAXDIST);
    R mat = PT_LIT(R, 0.0);
    uint32_t bits = set1 & ((S.meta.nplug >= 32) ? 0xFFFFFFFFu : ((1u << S.meta.nplug) - 1u));
    while (bits) {
        const int i = __ffs(bits) - 1;
        bits &= bits - 1u;
        const pt_sdf_plugin pl = S.plug[i];
        if (pl.kind != PT_SDF_NONE) {
            const V3<R> q = p - sdf_pos<R>(S, i);
            const R di = plugin_sdf(pl.kind, S.meta.custom_base + i, q);
            mat = (sdf < di) ? mat : plugin_material(pl, S.meta.custom_base + i, q);
            sdf = m_fmin(sdf, di);
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
template <typename V, typename R = SOf<V>> PT_DI R scene_sdf_material_hit(const KScene& S, V p, uint32_t set1, int hit_sel) {
    if (hit_sel >= 0) return plugin_material(S.plug[hit_sel], S.meta.custom_base + hit_sel, p - sdf_pos<R>(S, hit_sel));
    if (hit_sel == -1) return PT_LIT(R, 0.0);
    return scene_sdf_material(S, p, set1);
}

// RayIntersectAABB, SC:278-287.
template <typename V, typename R = SOf<V>> PT_DI V2<R> ray_aabb(V origin, V invdir, V pos, V size) {
    const V3<R> lo = origin - pos;
    const V3<R> tMin0 = fma3(size, v3<R>(-PT_LIT(R, 0.5), -PT_LIT(R, 0.5), -PT_LIT(R, 0.5)), -lo) * invdir;
    const V3<R> tMax0 = fma3(size, v3<R>(PT_LIT(R, 0.5), PT_LIT(R, 0.5), PT_LIT(R, 0.5)), -lo) * invdir;
    const V3<R> a = min3(tMin0, tMax0), b = max3(tMin0, tMax0);
    return v2<R>(m_fmax(m_fmax(a.x, a.y), a.z), m_fmin(m_fmin(b.x, b.y), b.z));
}

// SearchSDF, SC:732-777.
template <typename V, typename R = SOf<V>>
PT_DI bool search_sdf(const KScene& S, V p, V invdir, V2<R>& tMinMax, uint32_t& set1) {
    bool found = false;
    set1 = 0;
    const int n = S.meta.n[5];
    for (int i = 0; i < n; i++) {
        const V3<R> pos = sdf_pos<R>(S, i);
        const V3<R> size = v3<R>(S.sdfs[6 * i + 3], S.sdfs[6 * i + 4], S.sdfs[6 * i + 5]);
        const V2<R> bm = ray_aabb(p, invdir, pos, size);
        const uint32_t bit = 1u << i;  // n <= 32 is enforced on upload
        if ((bm.x > bm.y) || (bm.y < PT_LIT(R, 0.0))) continue;
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
template <typename R> PT_DI bool sphere_trace(const KScene& S, V3<R> org, V3<R> dir, HitT<R>& h) {
    R t = PT_LIT(R, 1e-3);
    R insT = PT_LIT(R, 0.0);
    const R omegaMax = PT_LIT(R, 1.70);
    const R omegaSpeed = PT_LIT(R, 0.20);
    R omega = omegaMax;
    R previousRadius = PT_LIT(R, 0.0);
    const V3<R> invdir = v3<R>(PT_LIT(R, 1.0) / dir.x, PT_LIT(R, 1.0) / dir.y, PT_LIT(R, 1.0) / dir.z);
    int points = 0;
    V2<R> tMinMax = v2<R>(R(PT_MAXDIST), R(PT_MAXDIST));
    uint32_t set1 = 0;
    V3<R> p;
    if (search_sdf(S, org, invdir, tMinMax, set1)) {
        t = m_fmax(tMinMax.x, t);
        p = fma3s(dir, t, org);
    } else {
        return false;
    }
    const R k = sign_glsl(scene_sdf_cold(S, org, set1));
    int hit_sel = -2;  // >= -1 once the march converged (scene_sdf_material_hit)
    // The reference's limits (512 steps, |d| < 1e-4, no distance cap) or the
    // scene's PT_EXT_MARCH ones.
    const bool xm = (S.ext.flags & PT_EXT_MARCH) != 0;
    const int maxSteps = xm ? S.ext.march_max_steps : 512;
    const R eps = xm ? S.ext.march_epsilon : PT_LIT(R, 1e-4);
    const R tmax = xm ? S.ext.march_max_distance : __int_as_float(0x7f800000);
#pragma unroll 1
    for (int i = 0; i < maxSteps; i++) {
        if (t > tmax) return false;  // past the distance cap: no SDF hit
        int sel;
        const R radius = scene_sdf_sel(S, p, set1, sel);
        if (insT > (m_fabs(previousRadius) + m_fabs(radius))) {
            t -= insT;
            omega = PT_LIT(R, 1.0);
            insT = previousRadius * omega * k;
            t += insT;
            p = fma3s(dir, t, org);
            continue;
        }
        if (m_fabs(radius) < eps) {
            hit_sel = sel;
            break;
        }
        if (t > tMinMax.y) {
            points += 1;
        } else {
            points = 0;
        }
        if (points >= 2) {
            t = tMinMax.y + PT_LIT(R, 1e-3);
            tMinMax = v2<R>(R(PT_MAXDIST), R(PT_MAXDIST));
            if (search_sdf(S, fma3s(dir, t, org), invdir, tMinMax, set1)) {
                tMinMax.x += t;
                tMinMax.y += t;
                t = m_fmax(tMinMax.x, t);
                p = fma3s(dir, t, org);
                continue;
            }
            return false;
        }
        insT = radius * omega * k;
        t += insT;
        p = fma3s(dir, t, org);
        const R omegaSpeedFactor = m_fmin(radius / previousRadius, PT_LIT(R, 0.99));
        omega += omegaSpeed * (m_fmin(PT_LIT(R, 1.0) / (PT_LIT(R, 1.0) - omegaSpeedFactor), omegaMax) - omega);
        previousRadius = radius;
    }
    if (t < h.hitdist) {
        h.hitdist = t - PT_LIT(R, 1e-3);
        p = fma3s(dir, t, org);
        // CalculateNumericalSDFNormals, SC:721-730.
        const R e = PT_LIT(R, 1e-4);
        const R nx = scene_sdf_cold(S, v3<R>(p.x + e, p.y + PT_LIT(R, 0.0), p.z + PT_LIT(R, 0.0)), set1) -
                         scene_sdf_cold(S, v3<R>(p.x - e, p.y - PT_LIT(R, 0.0), p.z - PT_LIT(R, 0.0)), set1);
        const R ny = scene_sdf_cold(S, v3<R>(p.x + PT_LIT(R, 0.0), p.y + e, p.z + PT_LIT(R, 0.0)), set1) -
                         scene_sdf_cold(S, v3<R>(p.x - PT_LIT(R, 0.0), p.y - e, p.z - PT_LIT(R, 0.0)), set1);
        const R nz = scene_sdf_cold(S, v3<R>(p.x + PT_LIT(R, 0.0), p.y + PT_LIT(R, 0.0), p.z + e), set1) -
                         scene_sdf_cold(S, v3<R>(p.x - PT_LIT(R, 0.0), p.y - PT_LIT(R, 0.0), p.z - e), set1);
        h.normal = normalize3(v3<R>(nx, ny, nz));
        h.materialID = scene_sdf_material_hit(S, p, set1, hit_sel);
        h.lightID = -PT_LIT(R, 1.0);
        return true;
    }
    return false;
}

// The analytic part of Intersection (SC:862-923) and of the object loop of
// LightSourceVisibilityCheck (SC:1121-1201): objectID = index of the last
// object whose test hit, -1 for none.
template <int FEAT = PT_FEAT_ALL, typename R = float>
PT_DI void intersect_analytic(const KScene& S, V3<R> org, V3<R> dir, HitT<R>& h, int& objectID) {
    int id = -1;
    const int n0 = S.meta.n[0], n1 = S.meta.n[1], n2 = S.meta.n[2], n3 = S.meta.n[3], n4 = S.meta.n[4];
    int gi = 0;
#pragma unroll 1
    for (int i = 0; i < n0; i++, gi++) {
        const int b = 6 * i;
        const V3<R> pos = v3<R>(S.objects[b], S.objects[b + 1], S.objects[b + 2]);
        if (sphere_intersect(org, dir, pos, S.objects[b + 3], (R)((int)S.objects[b + 4] - 1),
                             (R)((int)S.objects[b + 5] - 1), h))
            id = gi;
    }
#pragma unroll 1
    for (int i = 0; i < n1; i++, gi++) {
        const int b = S.meta.offset[1] + 5 * i;
        const V3<R> pos = v3<R>(S.objects[b], S.objects[b + 1], S.objects[b + 2]);
        if (plane_intersect(org, dir, pos, (R)((int)S.objects[b + 3] - 1), (R)((int)S.objects[b + 4] - 1),
                            h))
            id = gi;
    }
    if constexpr ((FEAT & PT_FEAT_BOX) != 0) {
#pragma unroll 1
        for (int i = 0; i < n2; i++, gi++) {
            const int b = S.meta.offset[2] + 11 * i;
            const V3<R> pos = v3<R>(S.objects[b], S.objects[b + 1], S.objects[b + 2]);
            const V3<R> size = v3<R>(S.objects[b + 6], S.objects[b + 7], S.objects[b + 8]);
            if (!bounding_sphere(org, dir, pos, PT_LIT(R, 0.25) * dot3(size, size))) continue;
            if (box_intersect(org, dir, pos, size, s_rotation_r<R>(S, gi), (R)((int)S.objects[b + 9] - 1),
                              (R)((int)S.objects[b + 10] - 1), h))
                id = gi;
        }
    }
    if constexpr ((FEAT & PT_FEAT_LENS) != 0) {
#pragma unroll 1
        for (int i = 0; i < n3; i++, gi++) {
            const int b = S.meta.offset[3] + 12 * i;
            LensGeomT<R> L;
            L.pos = v3<R>(S.objects[b], S.objects[b + 1], S.objects[b + 2]);
            L.radius = S.objects[b + 6];
            L.focal = S.objects[b + 7];
            L.thickness = S.objects[b + 8];
            L.converging = S.objects[b + 9] != PT_LIT(R, 0.0);
            if (!bounding_sphere(org, dir, L.pos, lens_bounding_radius2(L.radius, L.focal, L.thickness, L.converging)))
                continue;
            L.rot = s_rotation_r<R>(S, gi);
            int isOutside = 1;
            if (lens_intersect(org, dir, L, (R)((int)S.objects[b + 10] - 1), (R)((int)S.objects[b + 11] - 1),
                               h, isOutside))
                id = gi;
        }
    }
    if constexpr ((FEAT & PT_FEAT_CYCLIDE) != 0) {
#pragma unroll 1
        for (int i = 0; i < n4; i++, gi++) {
            const int b = S.meta.offset[4] + 16 * i;
            const V3<R> pos = v3<R>(S.objects[b], S.objects[b + 1], S.objects[b + 2]);
            if (!bounding_sphere(org, dir, pos, S.objects[b + 13])) continue;
            if (cyclide_intersect(S, org, dir, b, s_rotation_r<R>(S, gi), h)) id = gi;
        }
    }
    objectID = id;
}

// Intersection (SC:862-934) / LightSourceVisibilityCheck's loop: the analytic
// objects, then sphere tracing of the SDFs (objectID -2 for an SDF hit).
template <int FEAT = PT_FEAT_ALL, typename R = float>
PT_DI void intersect_all(const KScene& S, V3<R> org, V3<R> dir, HitT<R>& h, int& objectID) {
    intersect_analytic<FEAT>(S, org, dir, h, objectID);
    if constexpr ((FEAT & PT_FEAT_SDF) != 0) {
        if (S.meta.n[5] > 0) {
            if (sphere_trace(S, org, dir, h)) objectID = -2;
        }
    }
}
