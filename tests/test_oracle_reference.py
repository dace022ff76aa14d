"""The oracle's restatements of single shader functions against the
reference's own shader source: each function of oracle/ref_shader.py's list is
cut out of the reference's src/shader.comp, translated and built for the CPU
(oracle/_ref/libref_shader.so), and must give the oracle's results bit for bit
on seeded random inputs (RNG streams, sampling, spectra, refraction, MIS, the
cubic and quartic solvers, the rotation matrix, smin).  Needs the reference
tree (skipped without it)."""
import ctypes
import os

import numpy as np
import pytest

from oracle import ref_shader

REFERENCE = ref_shader.reference_root()
N = 4000

pytestmark = pytest.mark.skipif(not os.path.exists(ref_shader.shader_path(REFERENCE)),
                                reason="the reference tree is not mounted")

F = ctypes.c_float
FP = ctypes.POINTER(ctypes.c_float)
U32P = ctypes.POINTER(ctypes.c_uint32)
IP = ctypes.POINTER(ctypes.c_int)


@pytest.fixture(scope="module")
def libs(built):
    from oracle import oracle

    return oracle.lib(), ref_shader.load(REFERENCE)


def _bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


def _fn(lib, name, res, args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = args
    return f


def _seeds(n=N, seed=1):
    return np.random.default_rng(seed).integers(0, 2**32, n, dtype=np.uint64).astype(np.uint32)


def test_rng_streams(libs):
    o, r = libs
    seeds = _seeds()
    a = _fn(o, "pto_pcg32", ctypes.c_uint32, [ctypes.c_uint32])
    b = _fn(r, "refsh_pcg32", ctypes.c_uint32, [ctypes.c_uint32])
    assert all(a(int(s)) == b(int(s)) for s in seeds)
    a = _fn(o, "pto_random_float", F, [U32P])
    b = _fn(r, "refsh_random_float", F, [U32P])
    for s in seeds[:500]:
        sa, sb = ctypes.c_uint32(int(s)), ctypes.c_uint32(int(s))
        for _ in range(4):  # a stream: the state carries over
            assert _bits(a(ctypes.byref(sa))) == _bits(b(ctypes.byref(sb)))
            assert sa.value == sb.value
    a = _fn(o, "pto_generate_seed", ctypes.c_uint32, [ctypes.c_uint32, ctypes.c_uint32] + [ctypes.c_int] * 4)
    b = _fn(r, "refsh_generate_seed", ctypes.c_uint32, [ctypes.c_uint32, ctypes.c_uint32] + [ctypes.c_int] * 4)
    rng = np.random.default_rng(2)
    for _ in range(N):
        x, y = int(rng.integers(0, 4096)), int(rng.integers(0, 4096))
        frame, spf = int(rng.integers(1, 10**6)), int(rng.integers(1, 257))
        k, w = int(rng.integers(0, spf)), int(rng.integers(1, 4097))
        assert a(x, y, frame, spf, k, w) == b(x, y, frame, spf, k, w)


@pytest.mark.parametrize("name,width", [("sample_disk", 2), ("sample_sphere", 3)])
def test_seeded_samplers(libs, name, width):
    o, r = libs
    a = _fn(o, f"pto_fn_{name}", None, [U32P, FP])
    b = _fn(r, f"refsh_{name}", None, [U32P, FP])
    for s in _seeds(N, 3):
        sa, sb = ctypes.c_uint32(int(s)), ctypes.c_uint32(int(s))
        oa, ob = (F * width)(), (F * width)()
        a(ctypes.byref(sa), oa)
        b(ctypes.byref(sb), ob)
        assert sa.value == sb.value and (_bits(list(oa)) == _bits(list(ob))).all()


def test_direction_samplers_and_pdfs(libs):
    o, r = libs
    rng = np.random.default_rng(4)
    hemi_a = _fn(o, "pto_fn_sample_hemisphere", None, [FP, U32P, FP])
    hemi_b = _fn(r, "refsh_sample_hemisphere", None, [FP, U32P, FP])
    cone_a = _fn(o, "pto_fn_sample_cone", None, [U32P, F, FP])
    cone_b = _fn(r, "refsh_sample_cone", None, [U32P, F, FP])
    for s in _seeds(N, 5):
        n = rng.normal(size=3).astype(np.float32)
        n /= np.float32(np.linalg.norm(n))
        nn = (F * 3)(*n)
        sa, sb = ctypes.c_uint32(int(s)), ctypes.c_uint32(int(s))
        oa, ob = (F * 3)(), (F * 3)()
        hemi_a(nn, ctypes.byref(sa), oa)
        hemi_b(nn, ctypes.byref(sb), ob)
        assert (_bits(list(oa)) == _bits(list(ob))).all()
        cmax = float(np.float32(rng.uniform(0.0, 1.0)))
        cone_a(ctypes.byref(sa), cmax, oa)
        cone_b(ctypes.byref(sb), cmax, ob)
        assert sa.value == sb.value and (_bits(list(oa)) == _bits(list(ob))).all()
    cos_a = _fn(o, "pto_fn_cosine_pdf", F, [F])
    cos_b = _fn(r, "refsh_cosine_pdf", F, [F])
    cpdf_a = _fn(o, "pto_fn_cone_pdf", F, [F, F])
    cpdf_b = _fn(r, "refsh_cone_pdf", F, [F, F])
    mis_a = _fn(o, "pto_fn_mis", F, [F, F])
    mis_b = _fn(r, "refsh_mis", F, [F, F])
    for c, cm, p1, p2 in rng.uniform(0.0, 1.0, (N, 4)).astype(np.float32):
        assert _bits(cos_a(float(c))) == _bits(cos_b(float(c)))
        assert _bits(cpdf_a(float(c), float(cm))) == _bits(cpdf_b(float(c), float(cm)))
        assert _bits(mis_a(float(p1), float(p2))) == _bits(mis_b(float(p1), float(p2)))


def test_wavelengths_and_spectra(libs):
    o, r = libs
    rng = np.random.default_rng(6)
    hero_a = _fn(o, "pto_fn_hero_wavelength", F, [F, F, U32P])
    hero_b = _fn(r, "refsh_hero_wavelength", F, [F, F, U32P])
    wl_a = _fn(o, "pto_fn_sample_wavelengths", None, [F, FP])
    wl_b = _fn(r, "refsh_sample_wavelengths", None, [F, FP])
    spd_a = _fn(o, "pto_fn_spd", None, [FP, F, F, ctypes.c_int, FP])
    spd_b = _fn(r, "refsh_spd", None, [FP, F, F, ctypes.c_int, FP])
    bb_a = _fn(o, "pto_blackbody", None, [FP, F, FP])
    bb_b = _fn(r, "refsh_blackbody", None, [FP, F, FP])
    pk_a = _fn(o, "pto_blackbody_peak", F, [F])
    pk_b = _fn(r, "refsh_blackbody_peak", F, [F])
    n_a = _fn(o, "pto_bk7_index", F, [F])
    n_b = _fn(r, "refsh_bk7_index", F, [F])
    for s in _seeds(N, 7):
        sa, sb = ctypes.c_uint32(int(s)), ctypes.c_uint32(int(s))
        ha, hb = hero_a(360.0, 800.0, ctypes.byref(sa)), hero_b(360.0, 800.0, ctypes.byref(sb))
        assert _bits(ha) == _bits(hb) and sa.value == sb.value
        oa, ob = (F * 4)(), (F * 4)()
        wl_a(ha, oa)
        wl_b(ha, ob)
        assert (_bits(list(oa)) == _bits(list(ob))).all()
        lam = (F * 4)(*oa)
        peak, sig = float(np.float32(rng.uniform(380, 780))), float(np.float32(rng.uniform(1, 1000)))
        inv = int(rng.integers(0, 2))
        spd_a(lam, peak, sig, inv, oa)
        spd_b(lam, peak, sig, inv, ob)
        assert (_bits(list(oa)) == _bits(list(ob))).all()
        T = float(np.float32(rng.uniform(1000, 12000)))
        lm = (F * 4)(*[np.float32(v) * np.float32(1e-9) for v in lam])
        bb_a(lm, T, oa)
        bb_b(lm, T, ob)
        assert (_bits(list(oa)) == _bits(list(ob))).all()
        assert _bits(pk_a(T)) == _bits(pk_b(T))
        assert _bits(n_a(ha)) == _bits(n_b(ha))


def test_frames_smin_and_rotation(libs):
    o, r = libs
    rng = np.random.default_rng(8)
    tw_a = _fn(o, "pto_fn_to_world", None, [FP, FP, FP])
    tw_b = _fn(r, "refsh_to_world", None, [FP, FP, FP])
    sm_a = _fn(o, "pto_fn_smin", F, [F, F])
    sm_b = _fn(r, "refsh_smin", F, [F, F])
    sm2_a = _fn(o, "pto_fn_smin2", None, [FP, FP, FP])
    sm2_b = _fn(r, "refsh_smin2", None, [FP, FP, FP])
    rot_a = _fn(o, "pto_fn_rotation", None, [FP, FP])
    rot_b = _fn(r, "refsh_rotation", None, [FP, FP])
    for _ in range(N):
        n = rng.normal(size=3).astype(np.float32)
        n /= np.float32(np.linalg.norm(n))
        if rng.uniform() < 0.05:
            n = np.array([0.0, 0.0, -1.0], np.float32)  # the basis' special case
        v = rng.normal(size=3).astype(np.float32)
        oa, ob = (F * 3)(), (F * 3)()
        tw_a((F * 3)(*v), (F * 3)(*n), oa)
        tw_b((F * 3)(*v), (F * 3)(*n), ob)
        assert (_bits(list(oa)) == _bits(list(ob))).all()
        x, y = (float(t) for t in rng.uniform(-0.3, 0.3, 2).astype(np.float32))
        assert _bits(sm_a(x, y)) == _bits(sm_b(x, y))
        x2, y2 = rng.uniform(-0.3, 0.3, 2).astype(np.float32), rng.uniform(0, 4, 2).astype(np.float32)
        o2a, o2b = (F * 2)(), (F * 2)()
        sm2_a((F * 2)(x2[0], y2[0]), (F * 2)(x2[1], y2[1]), o2a)
        sm2_b((F * 2)(x2[0], y2[0]), (F * 2)(x2[1], y2[1]), o2b)
        assert (_bits(list(o2a)) == _bits(list(o2b))).all()
        ang = rng.uniform(-360, 360, 3).astype(np.float32)
        ma, mb = (F * 9)(), (F * 9)()
        rot_a((F * 3)(*ang), ma)
        rot_b((F * 3)(*ang), mb)
        assert (_bits(list(ma)) == _bits(list(mb))).all()


def test_polynomial_solvers(libs):
    o, r = libs
    rng = np.random.default_rng(9)
    c_a = _fn(o, "pto_fn_solve_cubic", ctypes.c_int, [F, F, F, FP])
    c_b = _fn(r, "refsh_solve_cubic", ctypes.c_int, [F, F, F, FP])
    q_a = _fn(o, "pto_fn_solve_quartic", None, [F] * 5 + [FP, IP])
    q_b = _fn(r, "refsh_solve_quartic", None, [F] * 5 + [FP, IP])
    ones = 0
    for _ in range(N):
        b, c, d = (float(v) for v in rng.normal(0, 3, 3).astype(np.float32))
        ra, rb = (F * 3)(), (F * 3)()
        na, nb = c_a(b, c, d, ra), c_b(b, c, d, rb)
        assert na == nb
        ones += na == 1
        assert (_bits(list(ra)[:na]) == _bits(list(rb)[:na])).all()
        a, b, c, d, e = (float(v) for v in rng.normal(0, 2, 5).astype(np.float32))
        if abs(a) < 1e-3:
            a = 1.0
        qa, qb = (F * 4)(), (F * 4)()
        fa, fb = (ctypes.c_int * 4)(), (ctypes.c_int * 4)()
        q_a(a, b, c, d, e, qa, fa)
        q_b(a, b, c, d, e, qb, fb)
        assert list(fa) == list(fb)
        real = np.array(list(fa), bool)
        assert (_bits(np.array(list(qa))[real]) == _bits(np.array(list(qb))[real])).all()
    assert 0 < ones < N  # both branches of the cubic ran


def _ray(rng):
    o = rng.uniform(-3.0, 3.0, 3)
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    if rng.uniform() < 0.3:  # aim near the object at the origin region
        d = -o / np.linalg.norm(o) + rng.normal(0, 0.2, 3)
        d /= np.linalg.norm(d)
    return (F * 6)(*np.concatenate([o, d]).astype(np.float32))


def _hit(rng):
    return [float(np.float32(1e5 if rng.uniform() < 0.7 else rng.uniform(0.5, 6.0))), 0.0, 0.0, 0.0, 0.0, -1.0]


def _same(fa, fb, ray, obj, rng, extra=False):
    h0 = _hit(rng)
    ha, hb = (F * 6)(*h0), (F * 6)(*h0)
    if extra:
        oa, ob = ctypes.c_int(1), ctypes.c_int(1)
        ra, rb = fa(ray, obj, ha, ctypes.byref(oa)), fb(ray, obj, hb, ctypes.byref(ob))
        assert oa.value == ob.value
    else:
        ra, rb = fa(ray, obj, ha), fb(ray, obj, hb)
    assert ra == rb
    assert (_bits(list(ha)) == _bits(list(hb))).all()
    return ra


@pytest.mark.parametrize("kind", ["sphere", "plane", "box", "lens", "cyclide"])
def test_intersections(libs, kind):
    """SphereIntersection, PlaneIntersection, BoxIntersection (with
    RotationMatrix), LensIntersection (two sphere slices) and DupinCyclide
    (the quartic solver): hit flag, distance, normal and ids bit for bit."""
    o, r = libs
    rng = np.random.default_rng(10)
    extra = kind == "lens"
    args = [FP, FP, FP] + ([IP] if extra else [])
    fa = _fn(o, f"pto_fn_{kind}", ctypes.c_int, args)
    fb = _fn(r, f"refsh_{kind}", ctypes.c_int, args)
    hits = 0
    for _ in range(N):
        pos = rng.uniform(-1.0, 1.0, 3)
        rot = rng.uniform(-180.0, 180.0, 3)
        ids = [float(rng.integers(1, 6)), float(rng.integers(0, 3))]
        if kind == "sphere":
            obj = [*pos, rng.uniform(0.1, 1.5), *ids]
        elif kind == "plane":
            obj = [*pos, *ids]
        elif kind == "box":
            obj = [*pos, *rot, *rng.uniform(0.2, 2.0, 3), *ids]
        elif kind == "lens":
            radius = rng.uniform(0.2, 1.0)
            obj = [*pos, *rot, radius, rng.uniform(0.6 * radius, 3.0), rng.uniform(0.0, 0.2),
                   float(rng.integers(0, 2)), *ids]
        else:
            a = rng.uniform(0.8, 1.2)
            obj = [*pos, *rot, *rng.uniform(0.5, 1.5, 3), a, rng.uniform(0.6, 0.95) * a, rng.uniform(0.2, 0.6),
                   rng.uniform(0.3, 0.6), 3.0, *ids]
        hits += _same(fa, fb, _ray(rng), (F * len(obj))(*np.asarray(obj, np.float32)), rng, extra)
    assert N // 50 < hits < N  # both outcomes ran


def test_bounds(libs):
    """BoundingSphere and RayIntersectAABB (with SortMinMax)."""
    o, r = libs
    rng = np.random.default_rng(11)
    bs_a = _fn(o, "pto_fn_bounding_sphere", ctypes.c_int, [FP, FP, F])
    bs_b = _fn(r, "refsh_bounding_sphere", ctypes.c_int, [FP, FP, F])
    ab_a = _fn(o, "pto_fn_aabb", None, [FP, FP, FP, FP, FP])
    ab_b = _fn(r, "refsh_aabb", None, [FP, FP, FP, FP, FP])
    for _ in range(N):
        ray = _ray(rng)
        pos = (F * 3)(*rng.uniform(-1.0, 1.0, 3).astype(np.float32))
        r2 = float(np.float32(rng.uniform(0.01, 4.0)))
        assert bs_a(ray, pos, r2) == bs_b(ray, pos, r2)
        d = np.array(list(ray)[3:], np.float32)
        inv = (F * 3)(*(np.float32(1.0) / d))
        size = (F * 3)(*rng.uniform(0.2, 2.0, 3).astype(np.float32))
        oa, ob = (F * 2)(), (F * 2)()
        ab_a(ray, inv, pos, size, oa)
        ab_b(ray, inv, pos, size, ob)
        assert (_bits(list(oa)) == _bits(list(ob))).all()
