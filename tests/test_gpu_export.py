"""SaveRender's tonemap chain on the device (pt_export_rgb8_device,
pt_read_rgb8) gives the same bytes as the host export (pt_export_rgb8) for
every tonemap, ragged sizes and unaligned output."""
import os

import numpy as np
import pytest

from conftest import SCENES

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env(built):
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no GPU")
    from pathtracer_gb300 import Context, Scene, cie_analytic, export_rgb8, native

    return torch, Context, Scene, cie_analytic(), export_rgb8, native


@pytest.mark.parametrize("W,H", [(23, 37), (64, 16), (1, 1)])
def test_device_export_matches_host(env, W, H):
    torch, _, _, _, export_rgb8, native = env
    rng = np.random.default_rng(W * 131 + H)
    acc = np.ones((H, W, 4), np.float32)
    acc[..., :3] = rng.uniform(-0.2, 4.0, (H, W, 3)).astype(np.float32)
    acc.reshape(-1, 4)[::7, :3] = 0.0
    d_acc = torch.from_numpy(acc).cuda()
    for offset in (0, 1):  # word stores and the byte path
        d_rgb = torch.zeros(H * W * 3 + 8, dtype=torch.uint8, device="cuda")
        for tm in range(4):
            rc = native.cuda().pt_export_rgb8_device(d_acc.data_ptr(), W, H, tm, d_rgb.data_ptr() + offset,
                                                    torch.cuda.current_stream().cuda_stream)
            assert rc == native.PT_OK
            torch.cuda.synchronize()
            got = d_rgb[offset:offset + H * W * 3].cpu().numpy().reshape(H, W, 3)
            assert np.array_equal(got, export_rgb8(acc, tm)), (tm, offset)
    assert native.cuda().pt_export_rgb8_device(d_acc.data_ptr(), W, H, 4, d_rgb.data_ptr(), None) == \
        native.PT_ERR_INVALID


def test_read_rgb8_of_a_render(env):
    _, Context, Scene, cie, export_rgb8, native = env
    scene = Scene.load(os.path.join(SCENES, "cornell_box.json"))
    W, H = 48, 40
    with Context(0) as ctx:
        ctx.bind(scene, cie)
        ctx.resize_accum(W, H)
        ctx.dispatch(scene.push_constants(W, H, 4, 4, 4, 8))
        ctx.wait()
        acc = ctx.read_accum()
        for tm in range(4):
            assert np.array_equal(ctx.read_rgb8(tm), export_rgb8(acc, tm))
