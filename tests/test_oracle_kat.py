"""Known-answer values of the CPU restatement, derived from the reference's
formulas (src/shader.comp).  The reference has no tests or golden vectors of
its own, so these pin the primitives the rest of the parity builds on."""
import ctypes
import math

import numpy as np
import pytest


@pytest.fixture(scope="module")
def L(built):
    from oracle import oracle

    return oracle.lib()


def test_pcg32_hash(L):
    # SC:937-941: state = seed*747796405 + 2891336453; RXS-M-XS output.
    assert L.pto_pcg32(0) == 129708002
    assert L.pto_pcg32(1) == 2831084092

    def ref(seed):
        state = (seed * 747796405 + 2891336453) & 0xFFFFFFFF
        word = (((state >> ((state >> 28) + 4)) ^ state) * 277803737) & 0xFFFFFFFF
        return ((word >> 22) ^ word) & 0xFFFFFFFF

    for s in [2, 12345, 0xFFFFFFFF, 0x80000000, 987654321]:
        assert L.pto_pcg32(s) == ref(s)


def test_random_float_is_seed_over_2_pow_32(L):
    # SC:943-946: float(seed) / float(0xFFFFFFFFu); 0xFFFFFFFF rounds to 2^32.
    s = ctypes.c_uint32(0)
    r = L.pto_random_float(ctypes.byref(s))
    assert s.value == 129708002
    assert r == np.float32(np.float32(129708002) / np.float32(4294967296.0))
    # a seed whose hash is >= 0xFFFFFF80 yields exactly 1.0
    assert L.pto_pcg32(60418823) == 0xFFFFFF90
    s = ctypes.c_uint32(60418823)
    assert L.pto_random_float(ctypes.byref(s)) == 1.0


def test_generate_seed(L):
    # SC:948-958: PCG32(frame - spf + k) + x + W*y (y already flipped).
    assert L.pto_generate_seed(0, 1, 1, 1, 0, 256) == 129708258
    assert L.pto_generate_seed(5, 7, 40, 8, 3, 100) == (L.pto_pcg32(35) + 5 + 700) & 0xFFFFFFFF


def test_bk7_sellmeier(L):
    # SC:1064-1073: BK7 at the helium d-line.
    assert abs(L.pto_bk7_index(587.56) - 1.51680) < 2e-5
    assert abs(L.pto_bk7_index(486.13) - 1.52238) < 2e-5


def test_blackbody_normalised_peak(L):
    # Planck / BlackBodyRadiationPeak is 1 at Wien's wavelength (SC:1040-1048).
    for T in (3000.0, 5500.0, 6500.0, 9000.0):
        lw = 2.897771955e-3 / T
        out = (ctypes.c_float * 4)()
        L.pto_blackbody((ctypes.c_float * 4)(lw, lw, lw, lw), ctypes.c_float(T), out)
        assert abs(out[0] / L.pto_blackbody_peak(T) - 1.0) < 1e-4


def test_sdf_plugins_known_values(L):
    from pathtracer_gb300 import native

    p = (ctypes.c_float * 3)
    blob = native.plugin(native.PT_SDF_BLOB, 0, (4, 5, 6))
    bulb = native.plugin(native.PT_SDF_MANDELBULB, 0, (4, 3, 0))
    menger = native.plugin(native.PT_SDF_MENGER, 1, (0, 0, 0))
    terrain = native.plugin(native.PT_SDF_TERRAIN, 1, (0, 0, 0))
    ev = lambda pl, *xyz: L.pto_sdf_eval(ctypes.byref(pl), p(*xyz))
    mat = lambda pl, *xyz: L.pto_sdf_material(ctypes.byref(pl), p(*xyz))
    # blob: far from the lobes the union is the unit sphere minus smin's blend.
    assert abs(ev(blob, 0.0, -3.0, 0.0) - 2.0) < 1e-6
    # mandelbulb: z <- r^8 (sin 8t sin 8f, cos 8f, cos 8t sin 8f) + p in float64, with t the
    # azimuth about y and f the polar angle from y (the Chebyshev form of the snippet).
    def bulb64(x, y, z):
        px, py, pz = x, y, z
        r = math.sqrt(x * x + y * y + z * z)
        dr = 1.0
        for _ in range(4):
            dr = 8.0 * r**7 * dr + 1.0
            t, f = math.atan2(x, z), math.acos(y / r)
            r8 = r**8
            x, y, z = (r8 * math.sin(8 * t) * math.sin(8 * f) + px, r8 * math.cos(8 * f) + py,
                       r8 * math.cos(8 * t) * math.sin(8 * f) + pz)
            r = math.sqrt(x * x + y * y + z * z)
            if r > 16.0:
                break
        return 0.5 * math.log(r) * r / dr

    for q in [(3.0, 20.0, 4.0), (0.3, 0.9, 0.5), (-0.7, 0.2, 0.6), (1.1, -0.4, 0.2)]:
        want = bulb64(*q)
        assert abs(ev(bulb, *q) - want) <= 1e-4 * abs(want), q
    # on the y axis the snippet divides 0 by 0 (inversesqrt(0)): NaN, as in the reference.
    assert math.isnan(ev(bulb, 0.0, 20.0, 0.0))
    assert abs(mat(bulb, 0.0, 0.0, 0.0) - 4.0) < 1e-6  # mix(4, 3, 0)
    # menger: the unit-half-size cube's surface and outside distance.
    assert abs(ev(menger, 3.0, 0.0, 0.0) - 2.0) < 1e-6
    assert mat(menger, 0.5, 0.5, 0.5) == 0.0
    # terrain: p.y - (h(x) + h(z)) with h(0) = sin(1.25) + 0.25 sin 1 + 0.125 sin 2 + ...
    h0 = (math.sin(1.25) + 0.25 * math.sin(1.0) + 0.125 * math.sin(2.0) + 0.0625 * math.sin(1.0)
          + 0.03125 * math.sin(5.0))
    assert abs(ev(terrain, 0.0, 3.0, 0.0) - (3.0 - 2 * h0)) < 2e-6


def test_wave_to_xyz_interpolates(L):
    # SC:129-140: linear interpolation in the 1 nm table; outside [360, 800] -> 0.
    cie = np.arange(1323, dtype=np.float32)
    out = (ctypes.c_float * 3)()
    L.pto_wave_to_xyz(cie.ctypes.data, ctypes.c_float(361.25), out)
    assert list(out) == [3.75, 4.75, 5.75]
    L.pto_wave_to_xyz(cie.ctypes.data, ctypes.c_float(359.0), out)
    assert list(out) == [0.0, 0.0, 0.0]
