"""Physical checks of the full-form extensions in the oracle (CPU only).

The GPU kernels are checked against the oracle path by path
(test_gpu_fullform.py); these tests check the oracle's restatement of the
extensions against expectations that follow from the physics alone, so a
mistake shared by both sides would still show:
- a camera that sees only the sky (a blackbody environment) measures
  exposure x integral of CMF(l) x sky(l) over the wavelength range, with the
  analytic CMF, the extension range and the sky emission;
- a mirror sphere under that sky returns its reflectance times the sky;
- a non-absorbing glass sphere (Cauchy or Sellmeier, dispersive) returns the
  sky unchanged on average (Fresnel choice, transmission at one wavelength
  with 4x weight), up to the few paths cut by the path length;
- a scene with extensions all zero renders as the reference's method, bit
  for bit.
"""
import math

import numpy as np
import pytest

SKY_T, SKY_L = 5800.0, 1.0
ISO, APERTURE = 1600, 0.0025


def _scene(objects=None, materials=None, spectral=None, march=None):
    root = {
        "camera": {"numShots": 1, "position": [[0.0, 0.0, 3.0]], "angle": [[180.0, 0.0]], "ISO": ISO, "size": 0.036,
                   "apertureSize": APERTURE, "apertureDistance": 0.049, "lensRadius": 0.01, "lensFocalLength": 0.03,
                   "lensThickness": 0.0, "lensDistance": 0.05},
        "environment": {"temperature": SKY_T, "luminosity": SKY_L},
        "spectral": spectral or {"range": [380.0, 780.0], "cmf": "analytic"},
        "material": materials or [],
        "sphere": objects or [],
    }
    if march:
        root["march"] = march
    return root


def _render(root, W=48, H=48, spf=16, depth=8, trace=True):
    from oracle import oracle, pack

    sc = pack.RefScene(root)
    ubo = sc.pack_ubo(pack.cie_analytic())
    push = sc.push_constants(W, H, spf, spf, spf, depth)
    acc = np.zeros((H, W, 4), np.float32)
    tr = oracle.dispatch(ubo, push, [], acc, trace_depth=depth if trace else 0, ext=sc.pack_ext())
    return acc, tr


def _planck_norm(l_nm, T):
    """The shader's normalised Planck spectrum (Emit: B(l, T) / B at Wien's peak) in double."""
    l = l_nm * 1e-9
    b = 1.1910429724e-16 / l ** 5 / (math.exp(0.014387768775 / (l * T)) - 1.0)
    return b / (4.0956746759e-6 * T ** 5)


def _cmf(l):
    def g(x, mu, s1, s2):
        t = (x - mu) / (s1 if x < mu else s2)
        return math.exp(-0.5 * t * t)

    x = 1.056 * g(l, 599.8, 37.9, 31.0) + 0.362 * g(l, 442.0, 16.0, 26.7) - 0.065 * g(l, 501.1, 20.4, 26.2)
    y = 0.821 * g(l, 568.8, 46.9, 40.5) + 0.286 * g(l, 530.9, 16.3, 31.1)
    z = 1.217 * g(l, 437.0, 11.8, 36.0) + 0.681 * g(l, 459.0, 26.0, 13.8)
    return np.array([x, y, z])


def test_sky_only_matches_the_spectral_integral():
    acc, _ = _render(_scene(), W=128, H=128, spf=16, trace=False)
    ls = np.linspace(380.0, 780.0, 4001)
    integrand = np.array([_cmf(l) * _planck_norm(l, SKY_T) * SKY_L for l in ls])
    want = np.trapezoid(integrand, ls, axis=0) * APERTURE * APERTURE * ISO
    got = acc[..., :3].reshape(-1, 3).mean(axis=0)
    assert np.allclose(got, want, rtol=4e-3), (got, want)  # 262 K samples x 4 wavelengths


def _first_hit_colours(root, obj=0):
    """Per-sample colours of paths whose first bounce hit object `obj`, and of
    paths that saw only the sky, from the oracle's trace."""
    from pathtracer_gb300 import native

    _, (ev, nev, col) = _render(root, W=64, H=64, spf=16, depth=8)
    first = ev[:, 0] & native.PT_EV_HIT_MASK
    return col[first == obj], col[first == native.PT_EV_HIT_MISS], ev[first == obj]


def test_mirror_returns_its_reflectance_times_the_sky():
    from pathtracer_gb300 import native

    root = _scene(objects=[{"position": [0.0, 0.0, 0.0], "radius": 0.8, "materialID": 1, "lightID": 0}],
                  materials=[{"reflection": {"peakWavelength": 550.0, "sigma": 1000.0, "isInvert": False},
                              "bsdf": {"type": "mirror", "reflectance": 0.9}}])
    hit, sky, ev = _first_hit_colours(root)
    assert len(hit) > 10000 and len(sky) > 10000
    assert np.all(ev[:, 0] & native.PT_EV_SPECULAR)
    ratio = hit.mean(axis=0) / sky.mean(axis=0)
    assert np.allclose(ratio, 0.9, rtol=0.02), ratio


@pytest.mark.parametrize("bsdf", [{"type": "cauchy", "A": 1.5, "B": 0.0042},
                                  {"type": "sellmeier", "B": [1.04, 0.23, 1.01], "C": [0.006, 0.02, 103.6]}])
def test_glass_sphere_conserves_the_sky(bsdf):
    from pathtracer_gb300 import native

    root = _scene(objects=[{"position": [0.0, 0.0, 0.0], "radius": 0.8, "materialID": 1, "lightID": 0}],
                  materials=[{"reflection": {"peakWavelength": 550.0, "sigma": 1000.0, "isInvert": False},
                              "bsdf": bsdf}])
    hit, sky, ev = _first_hit_colours(root)
    assert len(hit) > 10000
    refr = np.count_nonzero(ev[:, 0] & native.PT_EV_REFRACT)
    refl = np.count_nonzero(ev[:, 0] & native.PT_EV_SPECULAR)
    assert refr + refl == len(ev) and 0.02 < refl / len(ev) < 0.2  # Fresnel: a few per cent reflect
    ratio = hit.mean(axis=0) / sky.mean(axis=0)
    assert np.allclose(ratio, 1.0, rtol=0.03), ratio


def test_flat_and_smooth_lambert_under_the_sky():
    """A Lambertian sphere of flat albedo a under a uniform sky (no lights, so
    no light samples): each bounce keeps a of the throughput, so the first-hit
    paths carry at most a times the sky and at least a^depth of it."""
    root = _scene(objects=[{"position": [0.0, 0.0, 0.0], "radius": 0.8, "materialID": 1, "lightID": 0}],
                  materials=[{"reflection": {"peakWavelength": 550.0, "sigma": 1000.0, "isInvert": False},
                              "bsdf": {"type": "flat", "albedo": 0.5}}])
    hit, sky, _ = _first_hit_colours(root)
    ratio = hit.mean(axis=0) / sky.mean(axis=0)
    # a convex sphere: the diffusely reflected ray always escapes, so exactly a
    assert np.allclose(ratio, 0.5, rtol=0.03), ratio
    root["material"][0]["bsdf"] = {"type": "smooth", "base": 0.2, "amplitude": 0.6, "center": 550.0, "width": 60.0}
    hit, sky, _ = _first_hit_colours(root)
    ratio = hit.mean(axis=0) / sky.mean(axis=0)
    assert np.all((ratio > 0.2) & (ratio < 0.8)), ratio
    assert ratio[1] > ratio[2]  # the bump at 550 nm lifts Y (green) above Z (blue)


def test_zero_extensions_are_the_reference_method():
    """Flags 0: the oracle's extension entry renders as its reference entry."""
    import os

    from conftest import SCENES
    from oracle import oracle, pack

    sc = pack.load_scene(os.path.join(SCENES, "feature_mix.json"))
    ubo = sc.pack_ubo(pack.cie_analytic())
    push = sc.push_constants(24, 16, 2, 2, 2, 6)
    plugins = oracle.plugins_for_sources(sc.sdf_sources())
    a = np.zeros((16, 24, 4), np.float32)
    b = np.zeros((16, 24, 4), np.float32)
    oracle.dispatch(ubo, push, plugins, a)
    zero = pack.PtoSceneExt()
    zero.march_max_steps = 7  # ignored without its flag
    oracle.lib().pto_dispatch_ext(ubo.ctypes.data, __import__("ctypes").addressof(zero),
                                  __import__("ctypes").addressof(push), oracle._plugin_array(plugins), len(plugins),
                                  b.ctypes.data, 0, 0, 24, 16, None, 0)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_march_limits():
    """PT_EXT_MARCH: a distance cap below an SDF's distance makes it vanish; a
    step cap of 1 counts the first step's position as the hit (the
    reference's rule for an exhausted march)."""
    import os

    from conftest import SCENES
    from oracle import oracle, pack

    sc = pack.load_scene(os.path.join(SCENES, "mandelbulb_plane.json"))
    ubo = sc.pack_ubo(pack.cie_analytic())
    push = sc.push_constants(32, 24, 2, 2, 2, 1)
    plugins = oracle.plugins_for_sources(sc.sdf_sources())
    from pathtracer_gb300 import native

    def first_hits(ext):
        acc = np.zeros((24, 32, 4), np.float32)
        ev, _, _ = oracle.dispatch(ubo, push, plugins, acc, trace_depth=1, ext=ext)
        return ev[:, 0] & native.PT_EV_HIT_MASK

    base = first_hits(None)
    assert np.count_nonzero(base == native.PT_EV_HIT_SDF) > 50
    x = pack.PtoSceneExt()
    x.flags = pack.EXT_MARCH
    x.march_max_steps, x.march_epsilon, x.march_max_distance = 512, 1e-4, 0.5
    assert np.count_nonzero(first_hits(x) == native.PT_EV_HIT_SDF) == 0
    x.march_max_distance = 1e9
    assert np.array_equal(first_hits(x), base)  # the reference's limits, spelled out
