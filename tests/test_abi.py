"""The C ABI: both libraries load without a GPU and export every function
their headers in include/ declare."""
import ctypes
import os
import re

from conftest import ROOT


def _declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\**\s*(pt_[a-z_0-9]+)\s*\(", text, flags=re.M)))


def test_headers_declare_the_api():
    cuda = _declared("pt_cuda.h")
    host = _declared("pt_host.h")
    assert {"pt_create", "pt_dispatch", "pt_wait", "pt_upload_scene", "pt_set_sdfs"} <= set(cuda)
    assert {"pt_scene_parse", "pt_scene_pack_ubo", "pt_render_offscreen", "pt_export_rgb8"} <= set(host)


def test_libraries_export_every_declared_symbol(built):
    for header, lib in (("pt_cuda.h", built["cuda"]), ("pt_host.h", built["host"])):
        so = ctypes.CDLL(lib)
        missing = [name for name in _declared(header) if not hasattr(so, name)]
        assert not missing, (header, missing)


def test_python_binding_covers_every_declared_symbol(built):
    from pathtracer_gb300 import native

    assert set(_declared("pt_cuda.h")) == {n for n, _, _ in native.CUDA_API}
    assert set(_declared("pt_host.h")) == {n for n, _, _ in native.HOST_API}


def test_struct_layouts():
    from pathtracer_gb300 import native

    assert ctypes.sizeof(native.PtPush) == 88  # PushConstantValues
    assert native.UBO_FLOATS * 4 == 16388  # UniformBufferObject
    assert native.UBO_OFFSETS["CIEXYZ1931"][0] + 1323 == native.UBO_FLOATS


def test_no_context_without_gpu_is_a_status_not_a_crash(built):
    """pt_create on a machine without a usable device returns an error code."""
    import torch

    if torch.cuda.is_available():
        return
    from pathtracer_gb300 import native

    h = ctypes.c_void_p()
    rc = native.cuda().pt_create(ctypes.byref(h), 0)
    assert rc in (native.PT_ERR_CUDA, native.PT_ERR_OOM) and not h.value
