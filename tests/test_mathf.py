"""include/pt_mathf.h: accuracy against float64 on the CPU, and bit-identical
results on the GPU (the property the per-sample parity rests on)."""
import numpy as np
import pytest


def _ulp(got, ref64):
    ref = ref64.astype(np.float32)
    sp = np.spacing(np.abs(ref)).astype(np.float64)
    return np.abs(got.astype(np.float64) - ref64) / sp


def _inputs():
    rng = np.random.default_rng(1234)
    sc = np.concatenate([rng.uniform(-10, 10, 100000), rng.uniform(-4000, 4000, 50000),
                         rng.uniform(-65536, 65536, 20000), rng.uniform(-1e-3, 1e-3, 10000)]).astype(np.float32)
    ex = np.concatenate([rng.uniform(-87, 88.7, 100000), rng.uniform(-1, 1, 50000)]).astype(np.float32)
    lg = np.concatenate([np.exp(rng.uniform(-87, 88, 100000)), rng.uniform(0.5, 2, 50000),
                         rng.uniform(1e-45, 1e-38, 2000)]).astype(np.float32)
    ac = np.concatenate([rng.uniform(-1, 1, 100000), [-1.0, 1.0, 0.5, -0.5, 0.0]]).astype(np.float32)
    return rng, sc, ex, lg, ac


def _atan_inputs(rng):
    return np.concatenate([rng.uniform(-4, 4, 100000), np.exp(rng.uniform(-20, 20, 50000)),
                           -np.exp(rng.uniform(-20, 20, 20000)), [0.0, 1.0, -1.0]]).astype(np.float32)


def _atan2_inputs(rng):
    y = np.concatenate([rng.uniform(-10, 10, 100000), rng.uniform(-1e-3, 1e-3, 20000)]).astype(np.float32)
    x = np.concatenate([rng.uniform(-10, 10, 100000), rng.uniform(-5, 5, 20000)]).astype(np.float32)
    return y, x


def test_accuracy_cpu(built):
    from oracle import oracle

    rng, sc, ex, lg, ac = _inputs()
    assert _ulp(oracle.mathf("sin", sc), np.sin(sc.astype(np.float64))).max() <= 2.0
    assert _ulp(oracle.mathf("cos", sc), np.cos(sc.astype(np.float64))).max() <= 2.0
    assert _ulp(oracle.mathf("exp", ex), np.exp(ex.astype(np.float64))).max() <= 2.0
    assert _ulp(oracle.mathf("log", lg), np.log(lg.astype(np.float64))).max() <= 2.0
    assert _ulp(oracle.mathf("acos", ac), np.arccos(ac.astype(np.float64))).max() <= 2.0
    assert _ulp(oracle.mathf("asin", ac), np.arcsin(ac.astype(np.float64))).max() <= 2.5
    at = _atan_inputs(rng)
    assert _ulp(oracle.mathf("atan", at), np.arctan(at.astype(np.float64))).max() <= 2.0
    ya, xa = _atan2_inputs(rng)
    assert _ulp(oracle.mathf("atan2", ya, xa), np.arctan2(ya.astype(np.float64), xa.astype(np.float64))).max() <= 3.0
    e2 = np.concatenate([rng.uniform(-126, 127.9, 100000), rng.uniform(-1, 1, 50000)]).astype(np.float32)
    assert _ulp(oracle.mathf("exp2", e2), np.exp2(e2.astype(np.float64))).max() <= 2.0
    assert _ulp(oracle.mathf("log2", lg), np.log2(lg.astype(np.float64))).max() <= 3.0
    # pow on the shader's uses: r^7 (mandelbulb), l^-5 and T^5 (Planck), |u|^(1/3)
    # (cubic solver), 2^y (temporal accumulation weight).
    cases = [(rng.uniform(0, 16, 50000), 7.0), (rng.uniform(3e-7, 9e-7, 50000), -5.0),
             (rng.uniform(1e3, 2e4, 50000), 5.0), (np.exp(rng.uniform(-20, 20, 50000)), 0.3333333)]
    for x, y in cases:
        x = x.astype(np.float32)
        yy = np.full_like(x, y)
        assert _ulp(oracle.mathf("pow", x, yy), np.power(x.astype(np.float64), np.float64(np.float32(y)))).max() <= 8.0
    y2 = rng.uniform(-20, 0, 50000).astype(np.float32)
    assert _ulp(oracle.mathf("pow", np.full_like(y2, 2.0), y2), np.power(2.0, y2.astype(np.float64))).max() <= 8.0


def test_special_values_cpu(built):
    from oracle import oracle

    inf, nan = np.float32(np.inf), np.float32(np.nan)
    s = oracle.mathf("sin", np.array([0.0, -0.0, inf, nan], np.float32))
    assert s[0] == 0.0 and np.isnan(s[2]) and np.isnan(s[3])
    e = oracle.mathf("exp", np.array([0.0, 100.0, -200.0, -inf, inf, nan], np.float32))
    assert e[0] == 1.0 and e[1] == inf and e[2] == 0.0 and e[3] == 0.0 and e[4] == inf and np.isnan(e[5])
    lg = oracle.mathf("log", np.array([1.0, 0.0, -1.0, inf, nan], np.float32))
    assert lg[0] == 0.0 and lg[1] == -inf and np.isnan(lg[2]) and lg[3] == inf and np.isnan(lg[4])
    p = oracle.mathf("pow", np.array([-2.0, -2.0, 0.0, 0.0, 5.0, 1.0], np.float32),
                     np.array([3.0, 0.5, 2.0, -1.0, 0.0, nan], np.float32))
    assert p[0] == -8.0 and np.isnan(p[1]) and p[2] == 0.0 and p[3] == inf and p[4] == 1.0 and p[5] == 1.0
    a = oracle.mathf("acos", np.array([1.0, -1.0, 1.5], np.float32))
    assert a[0] == 0.0 and np.isnan(a[2])
    assert abs(float(a[1]) - np.pi) < 3e-7
    s = oracle.mathf("asin", np.array([0.0, -0.0, 1.0, -1.0, 1.5, nan], np.float32))
    assert s[0] == 0.0 and np.signbit(s[1]) and abs(float(s[2]) - np.pi / 2) < 2e-7 and s[3] == -s[2]
    assert np.isnan(s[4]) and np.isnan(s[5])
    t = oracle.mathf("atan", np.array([0.0, -0.0, inf, -inf, nan], np.float32))
    assert t[0] == 0.0 and np.signbit(t[1]) and abs(float(t[2]) - np.pi / 2) < 2e-7 and t[3] == -t[2]
    assert np.isnan(t[4])
    # atan2 at zeros and infinities (IEEE conventions), NaN in -> NaN out
    y = np.array([0.0, -0.0, 0.0, -0.0, 1.0, 1.0, -1.0, inf, inf, -inf, 1.0, nan], np.float32)
    x = np.array([0.0, 0.0, -0.0, -0.0, 0.0, -1.0, -inf, inf, -inf, 2.0, inf, 1.0], np.float32)
    r = oracle.mathf("atan2", y, x)
    ref = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    ok = np.isclose(r, ref, rtol=3e-7, atol=0) | (np.isnan(r) & np.isnan(ref))
    assert ok.all(), (r, ref)
    assert np.signbit(r[1]) == np.signbit(ref[1]) and np.signbit(r[3]) == np.signbit(ref[3])
    e = oracle.mathf("exp2", np.array([0.0, 1.0, -1.0, 10.0, 200.0, -200.0, -inf, nan], np.float32))
    assert list(e[:4]) == [1.0, 2.0, 0.5, 1024.0] and e[4] == inf and e[5] == 0.0 and e[6] == 0.0 and np.isnan(e[7])
    l2 = oracle.mathf("log2", np.array([1.0, 2.0, 0.5, 1024.0], np.float32))
    assert abs(float(l2[0])) == 0.0 and abs(float(l2[1]) - 1.0) < 2e-7 and abs(float(l2[2]) + 1.0) < 2e-7


@pytest.mark.gpu
def test_gpu_bits_equal_cpu(built):
    """Every function returns the same bits on the GPU as on the CPU."""
    import torch

    from oracle import oracle
    from pathtracer_gb300 import Context, native

    rng, sc, ex, lg, ac = _inputs()
    pw_x = np.concatenate([rng.uniform(0, 16, 20000), rng.uniform(3e-7, 9e-7, 20000),
                           np.exp(rng.uniform(-20, 20, 20000)), np.full(20000, 2.0)]).astype(np.float32)
    pw_y = np.concatenate([np.full(20000, 7.0), np.full(20000, -5.0), np.full(20000, 0.3333333),
                           rng.uniform(-20, 0, 20000)]).astype(np.float32)
    ya, xa = _atan2_inputs(rng)
    e2 = rng.uniform(-126, 127.9, 50000).astype(np.float32)
    cases = [("sin", sc, None), ("cos", sc, None), ("exp", ex, None), ("log", lg, None), ("acos", ac, None),
             ("pow", pw_x, pw_y), ("asin", ac, None), ("atan", _atan_inputs(rng), None), ("atan2", ya, xa),
             ("exp2", e2, None), ("log2", lg, None)]
    with Context(0) as ctx:
        for fn, x, y in cases:
            cpu = oracle.mathf(fn, x, y)
            dx = torch.from_numpy(x).cuda()
            dy = torch.from_numpy(y if y is not None else x).cuda()
            dout = torch.empty_like(dx)
            torch.cuda.synchronize()
            rc = native.cuda().pt_mathf_eval(ctx.handle, oracle.MATHF[fn], dx.data_ptr(), dy.data_ptr(),
                                             dout.data_ptr(), x.size)
            assert rc == 0, native.cuda().pt_last_error(ctx.handle)
            gpu = dout.cpu().numpy()
            same = (gpu.view(np.uint32) == cpu.view(np.uint32)) | (np.isnan(gpu) & np.isnan(cpu))
            assert same.all(), (fn, x[~same][:5], gpu[~same][:5], cpu[~same][:5])
