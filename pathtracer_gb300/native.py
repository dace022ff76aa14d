"""ctypes bindings of libpt_cuda (include/pt_cuda.h) and libpt_host
(include/pt_host.h).

This module only declares signatures and loads the in-tree libraries; it
never substitutes another implementation.  If a library is missing, loading
raises NativeLibraryError (call pathtracer_gb300.build.build() first).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib")

PT_OK = 0
PT_ERR_INVALID = 1
PT_ERR_CUDA = 2
PT_ERR_TIMEOUT = 3
PT_ERR_UNSUPPORTED = 4
PT_ERR_NO_SCENE = 5
PT_ERR_OOM = 6
PT_ERR_KERNEL = 7
PT_ERR_TOO_LARGE = 8
PT_ERR_BUSY = 9
PT_ERR_CANCELLED = 10
PT_NOALLOC_MAX_SAMPLES = 1 << 20

PT_ENGINE_MEGAKERNEL = 0
PT_ENGINE_WAVEFRONT = 1

PT_TARGET_FLOAT = 0
PT_TARGET_FP64 = 1

PT_BATCH_ROUTE_AUTO = 0
PT_BATCH_ROUTE_STAGED = 1
PT_BATCH_ROUTE_PERSISTENT = 2

PT_GEN_SPHERES = 0
PT_GEN_SDF = 1
PT_GEN_SDF_VARIED = 2
PT_GEN_SPHERES_FULL = 3

PT_SERVE_BATCHED = 0
PT_SERVE_PLAIN = 1

UBO_FLOATS = 4097  # 7 + 1024 + 768 + 783 + 128 + 64 + 1323
UBO_OFFSETS = {
    "numObjects": (0, 7),
    "objects": (7, 1024),
    "sdfs": (1031, 768),
    "materials": (1799, 783),
    "lights": (2582, 128),
    "lightIDs": (2710, 64),
    "CIEXYZ1931": (2774, 1323),
}

PT_SDF_NONE, PT_SDF_BLOB, PT_SDF_MANDELBULB, PT_SDF_MENGER, PT_SDF_TERRAIN, PT_SDF_CUSTOM = range(6)
PT_SDFMAT_DEFAULT, PT_SDFMAT_CONSTANT = 0, 1

PT_EV_HIT_MASK = 0xFFF
PT_EV_HIT_SDF = 0xFFE
PT_EV_HIT_MISS = 0xFFF
PT_EV_EMITTER = 1 << 12
PT_EV_LIGHT_SHIFT = 13
PT_EV_SHADOW_SHIFT = 20
PT_EV_RR_KILL = 1 << 22
PT_EV_VALID = 1 << 23


class NativeLibraryError(RuntimeError):
    pass


class PtPush(ctypes.Structure):
    """pt_push: byte-for-byte the reference's PushConstantValues (88 B)."""

    _fields_ = [
        ("resolution", ctypes.c_int32 * 2),
        ("frame", ctypes.c_int32),
        ("currentSamples", ctypes.c_int32),
        ("samplesPerFrame", ctypes.c_int32),
        ("FPS", ctypes.c_float),
        ("persistence", ctypes.c_float),
        ("pathLength", ctypes.c_int32),
        ("cameraAngle", ctypes.c_float * 2),
        ("cameraPosX", ctypes.c_float),
        ("cameraPosY", ctypes.c_float),
        ("cameraPosZ", ctypes.c_float),
        ("ISO", ctypes.c_int32),
        ("cameraSize", ctypes.c_float),
        ("apertureSize", ctypes.c_float),
        ("apertureDist", ctypes.c_float),
        ("lensRadius", ctypes.c_float),
        ("lensFocalLength", ctypes.c_float),
        ("lensThickness", ctypes.c_float),
        ("lensDistance", ctypes.c_float),
        ("tonemap", ctypes.c_int32),
    ]


class PtSdfPlugin(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("material_mode", ctypes.c_int32),
        ("material", ctypes.c_float * 3),
    ]


PT_EXT_SKY, PT_EXT_WAVELENGTHS, PT_EXT_ANALYTIC_CMF, PT_EXT_MARCH, PT_EXT_MATERIALS = 1, 2, 4, 8, 16
PT_BSDF_REFERENCE, PT_BSDF_FLAT, PT_BSDF_SMOOTH, PT_BSDF_MIRROR, PT_BSDF_CAUCHY, PT_BSDF_SELLMEIER = range(6)
PT_MAX_EXT_MATERIALS = 128
PT_EV_SPECULAR = 1 << 24
PT_EV_REFRACT = 1 << 25


class PtMaterialExt(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("p", ctypes.c_float * 6)]


class PtSceneExt(ctypes.Structure):
    """pt_scene_ext: a scene's full-form extensions (all zero: the reference's method)."""

    _fields_ = [
        ("flags", ctypes.c_int32),
        ("sky_temperature", ctypes.c_float),
        ("sky_luminosity", ctypes.c_float),
        ("lambda_min", ctypes.c_float),
        ("lambda_max", ctypes.c_float),
        ("march_max_steps", ctypes.c_int32),
        ("march_epsilon", ctypes.c_float),
        ("march_max_distance", ctypes.c_float),
        ("nmat", ctypes.c_int32),
        ("mat", PtMaterialExt * PT_MAX_EXT_MATERIALS),
    ]


class PtFrameState(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int32),
        ("height", ctypes.c_int32),
        ("frame", ctypes.c_int32),
        ("currentSamples", ctypes.c_int32),
        ("samplesPerFrame", ctypes.c_int32),
        ("FPS", ctypes.c_float),
        ("persistence", ctypes.c_float),
        ("pathLength", ctypes.c_int32),
        ("cameraShotIndex", ctypes.c_int32),
        ("tonemap", ctypes.c_int32),
    ]


class PtOffscreenOpts(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_int32),
        ("height", ctypes.c_int32),
        ("numSamples", ctypes.c_int32),
        ("samplesPerFrame", ctypes.c_int32),
        ("pathLength", ctypes.c_int32),
        ("cameraShotIndex", ctypes.c_int32),
        ("tonemap", ctypes.c_int32),
        ("frameOffset", ctypes.c_int32),
    ]


class PtWavefrontTuning(ctypes.Structure):
    _fields_ = [
        ("pool_slots", ctypes.c_uint32),
        ("march_budget", ctypes.c_int32),
        ("refill_min", ctypes.c_int32),
        ("drain_lanes", ctypes.c_int32),
        ("blocks_per_sm", ctypes.c_int32),
        ("march_inner", ctypes.c_int32),
    ]


class PtBatchInfo(ctypes.Structure):
    _fields_ = [
        ("samples_done", ctypes.c_uint64),
        ("samples_added", ctypes.c_uint64),
        ("iterations", ctypes.c_uint64),
        ("passes_added", ctypes.c_uint32),
        ("passes_pending", ctypes.c_uint32),
        ("pool_slots", ctypes.c_uint32),
        ("pass_slots", ctypes.c_uint32),
        ("passes_staged", ctypes.c_uint32),
        ("passes_persistent", ctypes.c_uint32),
        ("kernel_launches", ctypes.c_uint64),
    ]


class PtJobSpec(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("width", ctypes.c_int32),
        ("height", ctypes.c_int32),
        ("spp", ctypes.c_int32),
        ("pathLength", ctypes.c_int32),
        ("sdf_kind", ctypes.c_int32),
        ("objects", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("seed", ctypes.c_uint64),
    ]


class PtServerOpts(ctypes.Structure):
    _fields_ = [
        ("mode", ctypes.c_int32),
        ("spp_per_pass", ctypes.c_int32),
        ("hbm_budget", ctypes.c_uint64),
        ("pool_slots", ctypes.c_uint32),
        ("max_passes", ctypes.c_uint32),
        ("iterations_per_poll", ctypes.c_int32),
        ("passes_in_flight", ctypes.c_int32),
        ("keep_images", ctypes.c_int32),
        ("fp64_paths", ctypes.c_int32),
    ]


class PtServerJob(ctypes.Structure):
    _fields_ = [
        ("scene_key", ctypes.c_int32),
        ("max_spp", ctypes.c_int32),
        ("target_rmse", ctypes.c_double),
        ("push", PtPush),
    ]


class PtServerResult(ctypes.Structure):
    _fields_ = [
        ("job_id", ctypes.c_uint64),
        ("status", ctypes.c_int32),
        ("spp", ctypes.c_int32),
        ("rmse", ctypes.c_double),
        ("t_submit", ctypes.c_double),
        ("t_admit", ctypes.c_double),
        ("t_done", ctypes.c_double),
        ("samples", ctypes.c_uint64),
    ]


class PtServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_uint64),
        ("admitted", ctypes.c_uint64),
        ("completed", ctypes.c_uint64),
        ("samples", ctypes.c_uint64),
        ("bytes_in_use", ctypes.c_uint64),
        ("bytes_peak", ctypes.c_uint64),
        ("resident_bytes", ctypes.c_uint64),
        ("queued", ctypes.c_uint32),
        ("active", ctypes.c_uint32),
    ]


assert ctypes.sizeof(PtPush) == 88
assert ctypes.sizeof(PtSdfPlugin) == 20

_vp = ctypes.c_void_p
_i = ctypes.c_int
_sz = ctypes.c_size_t

# (name, restype, argtypes) for every symbol include/pt_cuda.h declares.
CUDA_API = [
    ("pt_create", _i, [ctypes.POINTER(_vp), _i]),
    ("pt_destroy", _i, [_vp]),
    ("pt_set_sdfs", _i, [_vp, ctypes.POINTER(ctypes.c_char_p), _i]),
    ("pt_set_sdf_plugins", _i, [_vp, ctypes.POINTER(PtSdfPlugin), _i]),
    ("pt_parse_sdf_source", _i, [ctypes.c_char_p, ctypes.POINTER(PtSdfPlugin)]),
    ("pt_upload_scene", _i, [_vp, _vp]),
    ("pt_upload_scene_ext", _i, [_vp, _vp, _vp]),
    ("pt_jit_check", _i, [ctypes.POINTER(ctypes.c_char_p), _i, _i, ctypes.c_char_p, _sz]),
    ("pt_glsl_translate", _i, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, _sz, ctypes.POINTER(_sz),
                               ctypes.c_char_p, _sz]),
    ("pt_resize_accum", _i, [_vp, _i, _i]),
    ("pt_dispatch", _i, [_vp, ctypes.POINTER(PtPush)]),
    ("pt_render_fp64", _i, [_vp, ctypes.POINTER(PtPush), _vp]),
    ("pt_wait", _i, [_vp, ctypes.c_uint64]),
    ("pt_read_accum", _i, [_vp, _vp, _sz]),
    ("pt_write_accum", _i, [_vp, _vp, _sz]),
    ("pt_accum_device_ptr", _vp, [_vp]),
    ("pt_export_rgb8_device", _i, [_vp, _i, _i, _i, _vp, _vp]),
    ("pt_read_rgb8", _i, [_vp, _i, _vp, _sz]),
    ("pt_stream", _vp, [_vp]),
    ("pt_set_stream", _i, [_vp, _vp]),
    ("pt_last_error", ctypes.c_char_p, [_vp]),
    ("pt_set_trace", _i, [_vp, _vp, _vp, _vp, _i]),
    ("pt_set_drain_limit", _i, [_vp, ctypes.c_uint64]),
    ("pt_set_device_checks", _i, [_vp, _i]),
    ("pt_set_fp_contract", _i, [_vp, _i]),
    ("pt_sdf_source_fingerprint", ctypes.c_uint64, [ctypes.c_char_p]),
    ("pt_mathf_eval", _i, [_vp, _i, _vp, _vp, _vp, _i]),
    ("pt_quartic_surface_eval", _i, [_vp, _i, _vp, _vp, _vp, _i]),
    ("pt_set_engine", _i, [_vp, _i]),
    ("pt_get_engine", _i, [_vp]),
    ("pt_set_wavefront_pool", _i, [_vp, ctypes.c_uint32]),
    ("pt_last_iterations", ctypes.c_uint32, [_vp]),
    ("pt_last_kernel_launches", ctypes.c_uint64, [_vp]),
    ("pt_set_wavefront_engines", _i, [_vp, _i]),
    ("pt_get_wavefront_engines", _i, [_vp]),
    ("pt_set_march_budget", _i, [_vp, _i]),
    ("pt_set_stage_timing", _i, [_vp, _i]),
    ("pt_get_stage_times", _i, [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64)]),
    ("pt_get_wavefront_tuning", _i, [_vp, ctypes.POINTER(PtWavefrontTuning)]),
    ("pt_set_wavefront_tuning", _i, [_vp, ctypes.POINTER(PtWavefrontTuning)]),
    ("pt_autotune_wavefront", _i, [_vp, ctypes.POINTER(PtPush), _i, ctypes.POINTER(PtWavefrontTuning),
                                   ctypes.POINTER(ctypes.c_double)]),
    ("pt_dispatch_noalloc", _i, [_vp, ctypes.POINTER(PtSdfPlugin), _i, ctypes.POINTER(PtPush), _vp, _vp]),
    ("pt_batch_create", _i, [ctypes.POINTER(_vp), _i, ctypes.c_uint32, ctypes.c_uint32]),
    ("pt_batch_destroy", _i, [_vp]),
    ("pt_batch_last_error", ctypes.c_char_p, [_vp]),
    ("pt_batch_stream", _vp, [_vp]),
    ("pt_batch_set_march_budget", _i, [_vp, _i]),
    ("pt_batch_set_route", _i, [_vp, _i]),
    ("pt_batch_set_device_checks", _i, [_vp, _i]),
    ("pt_batch_set_persist_refill", _i, [_vp, _i]),
    ("pt_batch_set_wavefront_engines", _i, [_vp, _i]),
    ("pt_batch_add_scene", _i, [_vp, _vp, ctypes.POINTER(PtSdfPlugin), _i, ctypes.POINTER(_i)]),
    ("pt_batch_set_scene_ext", _i, [_vp, _i, _vp]),
    ("pt_batch_add_scene_sources", _i, [_vp, _vp, ctypes.POINTER(ctypes.c_char_p), _i, ctypes.POINTER(_i)]),
    ("pt_batch_add_target", _i, [_vp, _i, _i, _i, ctypes.POINTER(_i)]),
    ("pt_batch_target_device_ptr", _vp, [_vp, _i]),
    ("pt_batch_add_pass", _i, [_vp, _i, _i, ctypes.POINTER(PtPush), ctypes.POINTER(_i)]),
    ("pt_batch_render_fp64", _i, [_vp, _i, _i, ctypes.POINTER(PtPush)]),
    ("pt_batch_step", _i, [_vp, _i, ctypes.POINTER(_i), _i, ctypes.POINTER(_i)]),
    ("pt_batch_pending", _i, [_vp]),
    ("pt_batch_run", _i, [_vp, ctypes.c_uint64]),
    ("pt_batch_stats", _i, [_vp, ctypes.POINTER(PtBatchInfo)]),
    ("pt_batch_target_samples", _i, [_vp, _i, ctypes.POINTER(ctypes.c_uint64)]),
    ("pt_batch_read_target", _i, [_vp, _i, _vp, _sz]),
    ("pt_batch_rmse", _i, [_vp, _i, _i, ctypes.POINTER(ctypes.c_double)]),
    ("pt_batch_rmse_many", _i, [_vp, ctypes.POINTER(_i), ctypes.POINTER(_i), _i, ctypes.POINTER(ctypes.c_double)]),
    ("pt_batch_rmse_image", _i, [_vp, _vp, _i, _i, _i, ctypes.POINTER(ctypes.c_double)]),
    ("pt_batch_release_target", _i, [_vp, _i]),
    ("pt_batch_release_scene", _i, [_vp, _i]),
]

# Every symbol include/pt_host.h declares.
HOST_API = [
    ("pt_scene_parse", _i, [ctypes.c_char_p, _sz, ctypes.POINTER(_vp), ctypes.c_char_p, _sz]),
    ("pt_scene_load_file", _i, [ctypes.c_char_p, ctypes.POINTER(_vp), ctypes.c_char_p, _sz]),
    ("pt_scene_free", None, [_vp]),
    ("pt_scene_counts", _i, [_vp, ctypes.POINTER(_i)]),
    ("pt_scene_pack_ubo", _i, [_vp, _vp, _vp]),
    ("pt_scene_pack_ext", _i, [_vp, _vp]),
    ("pt_scene_push_constants", _i, [_vp, ctypes.POINTER(PtFrameState), ctypes.POINTER(PtPush)]),
    ("pt_scene_sdf_source", ctypes.c_char_p, [_vp, _i]),
    ("pt_scene_to_json", _i, [_vp, ctypes.c_char_p, _sz, ctypes.POINTER(_sz)]),
    ("pt_scene_bind", _i, [_vp, _vp, _vp]),
    ("pt_render_offscreen", _i, [_vp, _vp, _vp, ctypes.POINTER(PtOffscreenOpts), _vp, _sz,
                                 ctypes.POINTER(ctypes.c_double)]),
    ("pt_export_rgb8", _i, [_vp, _i, _i, _i, _vp]),
    ("pt_save_ppm", _i, [ctypes.c_char_p, _vp, _i, _i]),
    ("pt_cie_analytic_table", None, [_vp]),
    ("pt_scene_sdf_plugins", _i, [_vp, ctypes.POINTER(PtSdfPlugin), _i, ctypes.POINTER(_i)]),
    ("pt_scene_generate", _i, [_i, ctypes.c_uint64, ctypes.POINTER(_vp), ctypes.POINTER(PtJobSpec)]),
    ("pt_server_create", _i, [ctypes.POINTER(_vp), _i, ctypes.POINTER(PtServerOpts)]),
    ("pt_server_destroy", _i, [_vp]),
    ("pt_server_last_error", ctypes.c_char_p, [_vp]),
    ("pt_server_now", ctypes.c_double, [_vp]),
    ("pt_server_set_mode", _i, [_vp, _i]),
    ("pt_server_batch", _vp, [_vp]),
    ("pt_server_add_scene", _i, [_vp, _i, _vp, ctypes.POINTER(PtSdfPlugin), _i]),
    ("pt_server_add_scene_sources", _i, [_vp, _i, _vp, ctypes.POINTER(ctypes.c_char_p), _i]),
    ("pt_server_render_reference", _i, [_vp, _i, ctypes.POINTER(PtPush), _i, _i]),
    ("pt_server_set_scene_ext", _i, [_vp, _i, _vp]),
    ("pt_server_submit", _i, [_vp, ctypes.POINTER(PtServerJob), ctypes.POINTER(ctypes.c_uint64)]),
    ("pt_server_poll", _i, [_vp, ctypes.POINTER(PtServerResult), _i, ctypes.POINTER(_i)]),
    ("pt_server_pending", _i, [_vp]),
    ("pt_server_read_image", _i, [_vp, ctypes.c_uint64, _vp, _sz]),
    ("pt_server_release", _i, [_vp, ctypes.c_uint64]),
    ("pt_server_cancel", _i, [_vp, ctypes.c_uint64]),
    ("pt_server_get_stats", _i, [_vp, ctypes.POINTER(PtServerStats)]),
    ("pt_server_run_trace", _i, [_vp, ctypes.POINTER(PtServerJob), ctypes.POINTER(ctypes.c_double), _i,
                                 ctypes.POINTER(PtServerResult)]),
]

_cache: dict[str, ctypes.CDLL] = {}


def _load(name: str, api) -> ctypes.CDLL:
    if name in _cache:
        return _cache[name]
    path = os.path.join(LIB_DIR, name)
    if not os.path.exists(path):
        raise NativeLibraryError(f"{path} is missing: build it with pathtracer_gb300.build.build()")
    lib = ctypes.CDLL(path)
    for sym, res, args in api:
        fn = getattr(lib, sym)
        fn.restype = res
        fn.argtypes = args
    _cache[name] = lib
    return lib


def cuda() -> ctypes.CDLL:
    """libpt_cuda.so (loads libcudart; no GPU needed until a context is made)."""
    return _load("libpt_cuda.so", CUDA_API)


def host() -> ctypes.CDLL:
    """libpt_host.so (links libpt_cuda.so)."""
    cuda()
    return _load("libpt_host.so", HOST_API)


def ptr(a: np.ndarray) -> int:
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data


def plugin(kind: int, mode: int = PT_SDFMAT_DEFAULT, material=(0.0, 0.0, 0.0)) -> PtSdfPlugin:
    p = PtSdfPlugin()
    p.kind = kind
    p.material_mode = mode
    for i, v in enumerate(material):
        p.material[i] = float(v)
    return p
