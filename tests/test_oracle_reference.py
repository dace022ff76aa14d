"""The oracle against the reference's own shader source (oracle/ref_shader.py
builds it for the CPU from the reference tree):
- single functions cut out of src/shader.comp (RNG streams, sampling,
  spectra, refraction, MIS, the cubic and quartic solvers, the rotation
  matrix, smin, the analytic intersections) give the oracle's results bit for
  bit on seeded random inputs;
- the whole shader without its interface and entry points, with a scene's
  SDF snippets spliced in as the reference's host does, gives the oracle's
  XYZ for every sample of the reference's own scene files, and the same
  Intersection() for rays into each scene.
Needs the reference tree (skipped without it)."""
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


@pytest.mark.parametrize("kind", ["sphere", "plane", "box", "lens", "cyclide", "thritorius", "smooth_cuboid"])
def test_intersections(libs, kind):
    """SphereIntersection, PlaneIntersection, BoxIntersection (with
    RotationMatrix), LensIntersection (two sphere slices), DupinCyclide (the
    quartic solver), and the two quartic surfaces the shader defines but
    never calls (Thritorius, SmoothCuboid): hit flag, distance, normal and
    ids bit for bit."""
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
        elif kind in ("thritorius", "smooth_cuboid"):
            obj = [0.0]  # fixed surfaces at the origin
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


# The reference's own scene files (whatever the checkout holds), and two of this repository's.
_SCENE_DIR = os.path.join(REFERENCE, "scenes")
REFERENCE_SCENES = sorted(f for f in os.listdir(_SCENE_DIR) if f.endswith(".json")) if os.path.isdir(_SCENE_DIR) else []
OWN_SCENES = ["cornell_box", "mandelbulb12_plane"]


def _scene_samples(lib, scene, W, H, spf, cie, plugins=()):
    """Per-sample XYZ of the reference's own Scene() (all pixels, all samples,
    in the oracle's trace order) and of the oracle."""
    from oracle import oracle

    ubo = scene.pack_ubo(cie)
    push = scene.push_constants(W, H, spf, spf, spf, 8)
    acc = np.zeros((H, W, 4), np.float32)
    _, _, col_o = oracle.dispatch(ubo, push, list(plugins), acc, trace_depth=16)
    lib.refsc_bind.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.refsc_scene.argtypes = [ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int, FP]
    lib.refsc_bind(ubo.ctypes.data, ctypes.addressof(push))
    col_r = np.zeros_like(col_o)
    out = (F * 3)()
    p = 0
    for y in range(H):
        for x in range(W):
            for k in range(spf):
                lib.refsc_scene(x, y, k, out)
                col_r[p] = list(out)
                p += 1
    return col_o, col_r


@pytest.mark.parametrize("name", REFERENCE_SCENES + OWN_SCENES)
def test_whole_shader_per_sample(built, name):
    """The reference's whole path tracer (src/shader.comp without its
    interface and `main`, built for the CPU over the shim, the scene buffer
    and push constants bound like the descriptor set, the scene's SDF
    snippets spliced in as the reference's host does) against the oracle on
    the reference's own scene files and two of this repository's (the
    Cornell box; the bench's 12-iteration mandelbulb, restated in C for the
    oracle): every sample's XYZ bit for bit, through lens refraction, NEE,
    MIS, Russian roulette, sphere tracing, SDF normals and SDF materials."""
    from conftest import SCENES
    from oracle import compare
    from pathtracer_gb300 import Scene, cie_analytic

    path = (os.path.join(SCENES, name + ".json") if name in OWN_SCENES
            else os.path.join(_SCENE_DIR, name))
    scene = Scene.load(path)
    texts = scene.sdf_sources()
    assert not any(t.startswith("builtin:") for t in texts)
    lib = ref_shader.load_scene(REFERENCE, texts)
    W, H, spf = (24, 16, 3) if not texts else (16, 12, 2)
    col_o, col_r = _scene_samples(lib, scene, W, H, spf, cie_analytic(), compare.plugins_for(scene))
    assert np.isfinite(col_o).all() and col_o.max() > 0
    bad = np.nonzero((_bits(col_o) != _bits(col_r)).any(axis=1))[0]
    assert bad.size == 0, (bad[:5], col_o[bad[:3]], col_r[bad[:3]])


@pytest.mark.parametrize("name", ["scene0.json", "scene3.json", "scene8.json", "scene9.json", "scene10.json"])
def test_whole_scene_intersection(built, name):
    """Intersection() of the reference's shader (analytic objects, then sphere
    tracing of the spliced SDFs) against the oracle's on rays aimed into the
    scene's SDF box (or at its origin): distance, normal and ids bit for bit."""
    from oracle import compare, oracle
    from pathtracer_gb300 import Scene, cie_analytic
    from pathtracer_gb300.native import PtSdfPlugin

    scene = Scene.load(os.path.join(REFERENCE, "scenes", name))
    ubo = scene.pack_ubo(cie_analytic())
    push = scene.push_constants(16, 12, 2, 2, 2, 8)
    plugins = compare.plugins_for(scene)
    arr = (PtSdfPlugin * max(1, len(plugins)))(*plugins)
    lib = ref_shader.load_scene(REFERENCE, scene.sdf_sources())
    lib.refsc_bind.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.refsc_intersection.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.refsc_bind(ubo.ctypes.data, ctypes.addressof(push))
    o = oracle.lib()
    o.pto_fn_intersection.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] + [ctypes.c_void_p] * 2
    box = ubo[7 + 1024:7 + 1024 + 6] if plugins else np.array([0, 0, 0, 2, 2, 2], np.float32)
    rng = np.random.default_rng(12)
    hits = 0
    for _ in range(1500):
        org = box[:3] + rng.uniform(-6.0, 6.0, 3)
        d = box[:3] + rng.uniform(-0.5, 0.5, 3) * box[3:] - org
        d /= np.linalg.norm(d)
        ray = (F * 6)(*np.concatenate([org, d]).astype(np.float32))
        a, b = (F * 6)(), (F * 6)()
        o.pto_fn_intersection(ubo.ctypes.data, ctypes.addressof(push), ctypes.addressof(arr), len(plugins), ray, a)
        lib.refsc_intersection(ray, b)
        assert (_bits(list(a)) == _bits(list(b))).all(), (list(a), list(b))
        hits += a[0] < 1e5
    assert hits > 100


@pytest.mark.parametrize("name", ["cornell_box", "scene9.json"])
def test_rendering_and_accumulate(built, name):
    """Rendering() and Accumulate() of the reference's shader (the samples of
    a dispatch, exposure, and the running mean or, on a reset frame, the
    exponential moving average) against the oracle's accumulator: three
    dispatches of a progressive render and one EMA frame, every pixel bit for
    bit."""
    from conftest import SCENES
    from oracle import compare, oracle
    from pathtracer_gb300 import Scene, cie_analytic

    path = (os.path.join(SCENES, "cornell_box.json") if name == "cornell_box"
            else os.path.join(REFERENCE, "scenes", name))
    scene = Scene.load(path)
    W, H, spf = 12, 8, 2
    lib = ref_shader.load_scene(REFERENCE, scene.sdf_sources())
    lib.refsc_bind.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.refsc_rendering.argtypes = [ctypes.c_uint32, ctypes.c_uint32, FP, FP]
    ubo = scene.pack_ubo(cie_analytic())
    plugins = compare.plugins_for(scene)
    acc_o = np.zeros((H, W, 4), np.float32)
    acc_r = np.zeros((H, W, 3), np.float32)
    # (frame, currentSamples): progressive frames, then a reset frame with frame > spf (the EMA branch)
    for frame, cur in ((spf, spf), (2 * spf, 2 * spf), (3 * spf, 3 * spf), (4 * spf, spf)):
        push = scene.push_constants(W, H, frame, cur, spf, 6)
        push.FPS, push.persistence = 30.0, 0.5
        oracle.dispatch(ubo, push, plugins, acc_o)
        lib.refsc_bind(ubo.ctypes.data, ctypes.addressof(push))
        out = (F * 3)()
        nxt = np.empty_like(acc_r)
        for y in range(H):
            for x in range(W):
                lib.refsc_rendering(x, y, (F * 3)(*acc_r[y, x]), out)
                nxt[y, x] = list(out)
        acc_r = nxt
        assert (_bits(acc_o[..., :3]) == _bits(acc_r)).all(), (frame, cur)
    assert acc_r.max() > 0
