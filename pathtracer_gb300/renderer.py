"""Python mirror of the drop-in boundary: a Context over libpt_cuda and a
Scene over libpt_host, with the reference host's calls by name.

    scene = Scene.load("pathtracer_gb300/scenes/mandelbulb_plane.json")
    with Context(device=0) as ctx:
        accum, secs = render_offscreen(ctx, scene, cie_analytic(), 1024, 1024, num_samples=64, spf=64, path_length=6)

Every call goes through the C ABI; a failing status raises PathTracerError
with the library's message.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native
from .native import PtFrameState, PtOffscreenOpts, PtPush


class PathTracerError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def cie_analytic() -> np.ndarray:
    """CIE 1931 table (1323 floats, 360..800 nm) from the Wyman-Sloan-Shirley fit."""
    out = np.zeros(1323, np.float32)
    native.host().pt_cie_analytic_table(native.ptr(out))
    return out


class Scene:
    """A parsed scene JSON (the reference's schema)."""

    def __init__(self, handle: int):
        self._h = ctypes.c_void_p(handle)
        self._lib = native.host()

    @classmethod
    def parse(cls, text: str | bytes) -> "Scene":
        data = text.encode() if isinstance(text, str) else text
        h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(512)
        rc = native.host().pt_scene_parse(data, len(data), ctypes.byref(h), err, 512)
        if rc != native.PT_OK:
            raise PathTracerError(rc, err.value.decode())
        return cls(h.value)

    @classmethod
    def load(cls, path: str) -> "Scene":
        with open(path, "rb") as f:
            return cls.parse(f.read())

    @classmethod
    def generate(cls, kind: int, seed: int) -> tuple["Scene", native.PtJobSpec]:
        """A seeded synthetic job (pt_scene_generate): the scene and its spec."""
        h = ctypes.c_void_p()
        spec = native.PtJobSpec()
        rc = native.host().pt_scene_generate(kind, ctypes.c_uint64(seed), ctypes.byref(h), ctypes.byref(spec))
        if rc != native.PT_OK:
            raise PathTracerError(rc, "pt_scene_generate failed")
        return cls(h.value), spec

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._lib.pt_scene_free(h)
            self._h = None

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def counts(self) -> dict[str, int]:
        c = (ctypes.c_int * 9)()
        self._lib.pt_scene_counts(self._h, c)
        keys = ["spheres", "planes", "boxes", "lenses", "cyclides", "sdfs", "materials", "lights", "shots"]
        return dict(zip(keys, list(c)))

    def pack_ubo(self, cie: np.ndarray | None) -> np.ndarray:
        ubo = np.zeros(native.UBO_FLOATS, np.float32)
        cie_p = None if cie is None else native.ptr(np.ascontiguousarray(cie, np.float32))
        rc = self._lib.pt_scene_pack_ubo(self._h, cie_p, native.ptr(ubo))
        if rc != native.PT_OK:
            raise PathTracerError(rc, "scene overflows the uniform buffer arrays")
        return ubo

    def pack_ext(self) -> native.PtSceneExt:
        """pt_scene_pack_ext: the scene's full-form extensions (flags 0: none)."""
        out = native.PtSceneExt()
        rc = self._lib.pt_scene_pack_ext(self._h, ctypes.byref(out))
        if rc != native.PT_OK:
            raise PathTracerError(rc, "scene extensions do not fit pt_scene_ext")
        return out

    def ext_or_none(self):
        """pack_ext(), or None for a scene of the reference's method."""
        x = self.pack_ext()
        return x if x.flags else None

    def push_constants(self, width: int, height: int, frame: int, current_samples: int, spf: int,
                       path_length: int, shot: int = 1, fps: float = 1.0 / 0.0166, persistence: float = 0.0625,
                       tonemap: int = 3) -> PtPush:
        st = PtFrameState(width, height, frame, current_samples, spf, fps, persistence, path_length, shot, tonemap)
        out = PtPush()
        rc = self._lib.pt_scene_push_constants(self._h, ctypes.byref(st), ctypes.byref(out))
        if rc != native.PT_OK:
            raise PathTracerError(rc, "bad frame state or camera shot index")
        return out

    def sdf_sources(self) -> list[str]:
        n = self.counts()["sdfs"]
        return [self._lib.pt_scene_sdf_source(self._h, i).decode() for i in range(n)]

    def sdf_plugins(self) -> list:
        n = self.counts()["sdfs"]
        arr = (native.PtSdfPlugin * max(1, n))()
        cnt = ctypes.c_int()
        rc = self._lib.pt_scene_sdf_plugins(self._h, arr, n, ctypes.byref(cnt))
        if rc != native.PT_OK:
            raise PathTracerError(rc, "an SDF source is not a recognised plug-in")
        return list(arr[:n])

    def to_json(self) -> str:
        need = ctypes.c_size_t()
        self._lib.pt_scene_to_json(self._h, None, 0, ctypes.byref(need))
        buf = ctypes.create_string_buffer(need.value)
        rc = self._lib.pt_scene_to_json(self._h, buf, need, ctypes.byref(need))
        if rc != native.PT_OK:
            raise PathTracerError(rc, "to_json failed")
        return buf.value.decode()


class Context:
    """pt_ctx: one device, one stream, owns the accumulator."""

    def __init__(self, device: int = 0):
        self._lib = native.cuda()
        h = ctypes.c_void_p()
        rc = self._lib.pt_create(ctypes.byref(h), device)
        if rc != native.PT_OK:
            raise PathTracerError(rc, f"pt_create(device={device}) failed")
        self._h = h
        self.width = self.height = 0

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.pt_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def _check(self, rc: int):
        if rc != native.PT_OK:
            raise PathTracerError(rc, self._lib.pt_last_error(self._h).decode())

    def set_sdfs(self, sources: list[str]):
        arr = (ctypes.c_char_p * max(1, len(sources)))(*[s.encode() for s in sources])
        self._check(self._lib.pt_set_sdfs(self._h, arr, len(sources)))

    def set_sdf_plugins(self, plugins: list):
        arr = (native.PtSdfPlugin * max(1, len(plugins)))(*plugins)
        self._check(self._lib.pt_set_sdf_plugins(self._h, arr, len(plugins)))

    def upload_scene(self, ubo: np.ndarray, ext=None):
        ubo = np.ascontiguousarray(ubo, np.float32)
        assert ubo.size == native.UBO_FLOATS
        if ext is None:
            self._check(self._lib.pt_upload_scene(self._h, native.ptr(ubo)))
        else:
            self._check(self._lib.pt_upload_scene_ext(self._h, native.ptr(ubo), ctypes.byref(ext)))

    def bind(self, scene: Scene, cie: np.ndarray):
        cie = np.ascontiguousarray(cie, np.float32)
        self._check(native.host().pt_scene_bind(self._h, scene.handle, native.ptr(cie)))

    def resize_accum(self, width: int, height: int):
        self._check(self._lib.pt_resize_accum(self._h, width, height))
        self.width, self.height = width, height

    def dispatch(self, push: PtPush):
        self._check(self._lib.pt_dispatch(self._h, ctypes.byref(push)))

    def render_fp64(self, push: PtPush, d_sums: int):
        """pt_render_fp64: the dispatch's paths in double precision, summed
        into the caller's device array of W*H*4 doubles (x, y, z, count)."""
        self._check(self._lib.pt_render_fp64(self._h, ctypes.byref(push), d_sums))

    def wait(self, timeout_ns: int = 2**64 - 1):
        self._check(self._lib.pt_wait(self._h, ctypes.c_uint64(timeout_ns)))

    def read_accum(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((self.height, self.width, 4), np.float32)
        self._check(self._lib.pt_read_accum(self._h, native.ptr(out), out.nbytes))
        return out

    def read_rgb8(self, tonemap: int = 3) -> np.ndarray:
        """The accumulator through SaveRender's tonemap chain on the device."""
        out = np.empty((self.height, self.width, 3), np.uint8)
        self._check(self._lib.pt_read_rgb8(self._h, tonemap, native.ptr(out), out.nbytes))
        return out

    def write_accum(self, data: np.ndarray):
        data = np.ascontiguousarray(data, np.float32)
        self._check(self._lib.pt_write_accum(self._h, native.ptr(data), data.nbytes))

    def accum_device_ptr(self) -> int:
        return self._lib.pt_accum_device_ptr(self._h) or 0

    def stream(self) -> int:
        return self._lib.pt_stream(self._h) or 0

    def set_stream(self, stream: int | None):
        self._check(self._lib.pt_set_stream(self._h, stream))

    def set_engine(self, engine: int):
        self._check(self._lib.pt_set_engine(self._h, engine))

    def engine(self) -> int:
        return self._lib.pt_get_engine(self._h)

    def set_wavefront_pool(self, slots: int):
        self._check(self._lib.pt_set_wavefront_pool(self._h, slots))

    def set_wavefront_engines(self, engines: int):
        """pt_set_wavefront_engines: engines (1..4, on streams of their own) a large dispatch is split between."""
        self._check(self._lib.pt_set_wavefront_engines(self._h, engines))

    def wavefront_engines(self) -> int:
        return self._lib.pt_get_wavefront_engines(self._h)

    def set_march_budget(self, steps: int):
        self._check(self._lib.pt_set_march_budget(self._h, steps))

    STAGES = ("isect", "march", "shade", "gen", "book")

    def set_stage_timing(self, on: bool):
        self._check(self._lib.pt_set_stage_timing(self._h, int(on)))

    def stage_times(self) -> tuple[dict, int]:
        """Device ms per wavefront stage since stage timing was switched on, and the iterations timed."""
        ms = (ctypes.c_double * 5)()
        it = ctypes.c_uint64()
        self._check(self._lib.pt_get_stage_times(self._h, ms, ctypes.byref(it)))
        return dict(zip(self.STAGES, list(ms))), it.value

    def tuning(self) -> dict:
        t = native.PtWavefrontTuning()
        self._check(self._lib.pt_get_wavefront_tuning(self._h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in native.PtWavefrontTuning._fields_}

    def set_tuning(self, **kw):
        cur = self.tuning()
        cur.update(kw)
        t = native.PtWavefrontTuning(**cur)
        self._check(self._lib.pt_set_wavefront_tuning(self._h, ctypes.byref(t)))

    def autotune(self, push: PtPush, rounds: int = 1) -> tuple[dict, float]:
        """pt_autotune_wavefront: installs and returns the fastest knobs."""
        t = native.PtWavefrontTuning()
        secs = ctypes.c_double()
        self._check(self._lib.pt_autotune_wavefront(self._h, ctypes.byref(push), rounds, ctypes.byref(t),
                                                    ctypes.byref(secs)))
        return {k: getattr(t, k) for k, _ in native.PtWavefrontTuning._fields_}, secs.value

    def last_iterations(self) -> int:
        return self._lib.pt_last_iterations(self._h)

    def last_kernel_launches(self) -> int:
        """Kernels the last dispatch launched."""
        return self._lib.pt_last_kernel_launches(self._h)

    def set_fp_contract(self, on: bool):
        """pt_set_fp_contract: FMA contraction in run-time compiled kernels (off: bit-exact)."""
        self._check(self._lib.pt_set_fp_contract(self._h, int(bool(on))))

    def set_drain_limit(self, max_iterations: int):
        """Caps the wavefront drain's iterations (0: the library's bound)."""
        self._check(self._lib.pt_set_drain_limit(self._h, max_iterations))

    def set_device_checks(self, on: bool):
        """The wavefront engine's kernels with index checks (pt_set_device_checks)."""
        self._check(self._lib.pt_set_device_checks(self._h, int(on)))

    def set_trace(self, events_ptr: int, nevents_ptr: int, colors_ptr: int, depth_cap: int):
        self._check(self._lib.pt_set_trace(self._h, events_ptr or None, nevents_ptr or None, colors_ptr or None,
                                           depth_cap))


class Batch:
    """pt_batch: many scenes, targets and passes in one wavefront pool."""

    def __init__(self, device: int = 0, pool_slots: int = 1 << 19, max_passes: int = 4096):
        self._lib = native.cuda()
        h = ctypes.c_void_p()
        rc = self._lib.pt_batch_create(ctypes.byref(h), device, pool_slots, max_passes)
        if rc != native.PT_OK:
            raise PathTracerError(rc, f"pt_batch_create(device={device}) failed")
        self._h = h
        self._sizes: dict[int, tuple[int, int]] = {}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.pt_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    @property
    def handle(self) -> ctypes.c_void_p:
        return self._h

    def _check(self, rc: int):
        if rc != native.PT_OK:
            raise PathTracerError(rc, self._lib.pt_batch_last_error(self._h).decode())

    def stream(self) -> int:
        return self._lib.pt_batch_stream(self._h) or 0

    def set_march_budget(self, steps: int):
        self._check(self._lib.pt_batch_set_march_budget(self._h, steps))

    def set_persist_refill(self, lanes: int):
        self._check(self._lib.pt_batch_set_persist_refill(self._h, lanes))

    def set_wavefront_engines(self, engines: int):
        """pt_batch_set_wavefront_engines: 1, or 2 staged engines that split large passes."""
        self._check(self._lib.pt_batch_set_wavefront_engines(self._h, engines))

    def set_route(self, route: int):
        self._check(self._lib.pt_batch_set_route(self._h, route))

    def set_device_checks(self, on: bool):
        """Both engines' kernels with index checks (pt_batch_set_device_checks)."""
        self._check(self._lib.pt_batch_set_device_checks(self._h, int(on)))

    def add_scene(self, ubo: np.ndarray, plugins: list) -> int:
        ubo = np.ascontiguousarray(ubo, np.float32)
        assert ubo.size == native.UBO_FLOATS
        arr = (native.PtSdfPlugin * max(1, len(plugins)))(*plugins)
        out = ctypes.c_int()
        self._check(self._lib.pt_batch_add_scene(self._h, native.ptr(ubo), arr, len(plugins), ctypes.byref(out)))
        return out.value

    def set_scene_ext(self, scene_id: int, ext):
        """pt_batch_set_scene_ext (ext None: the reference's method)."""
        self._check(self._lib.pt_batch_set_scene_ext(self._h, scene_id, ctypes.byref(ext) if ext is not None else None))

    def add_scene_sources(self, ubo: np.ndarray, sources: list[str]) -> int:
        """pt_batch_add_scene_sources: SDFs as text (shipped snippets or any GLSL)."""
        ubo = np.ascontiguousarray(ubo, np.float32)
        assert ubo.size == native.UBO_FLOATS
        arr = (ctypes.c_char_p * max(1, len(sources)))(*[t.encode() for t in sources])
        out = ctypes.c_int()
        self._check(self._lib.pt_batch_add_scene_sources(self._h, native.ptr(ubo), arr, len(sources),
                                                          ctypes.byref(out)))
        return out.value

    def add_target(self, width: int, height: int, kind: int = native.PT_TARGET_FLOAT) -> int:
        out = ctypes.c_int()
        self._check(self._lib.pt_batch_add_target(self._h, width, height, kind, ctypes.byref(out)))
        self._sizes[out.value] = (width, height)
        return out.value

    def add_pass(self, scene: int, target: int, push: PtPush) -> int:
        out = ctypes.c_int()
        self._check(self._lib.pt_batch_add_pass(self._h, scene, target, ctypes.byref(push), ctypes.byref(out)))
        return out.value

    def render_fp64(self, scene: int, target: int, push: PtPush):
        """pt_batch_render_fp64: one dispatch's samples traced in double
        precision into an FP64 target."""
        self._check(self._lib.pt_batch_render_fp64(self._h, scene, target, ctypes.byref(push)))

    def step(self, iterations: int, capacity: int = 4096) -> list[int]:
        ids = (ctypes.c_int * max(1, capacity))()
        n = ctypes.c_int()
        self._check(self._lib.pt_batch_step(self._h, iterations, ids, capacity, ctypes.byref(n)))
        return list(ids[: n.value])

    def pending(self) -> int:
        return self._lib.pt_batch_pending(self._h)

    def run(self, max_iterations: int = 1 << 40):
        self._check(self._lib.pt_batch_run(self._h, ctypes.c_uint64(max_iterations)))

    def stats(self) -> dict:
        info = native.PtBatchInfo()
        self._check(self._lib.pt_batch_stats(self._h, ctypes.byref(info)))
        return {k: getattr(info, k) for k, _ in native.PtBatchInfo._fields_}

    def target_samples(self, target: int) -> int:
        out = ctypes.c_uint64()
        self._check(self._lib.pt_batch_target_samples(self._h, target, ctypes.byref(out)))
        return out.value

    def read_target(self, target: int) -> np.ndarray:
        w, h = self._sizes[target]
        out = np.empty((h, w, 4), np.float32)
        self._check(self._lib.pt_batch_read_target(self._h, target, native.ptr(out), out.nbytes))
        return out

    def target_device_ptr(self, target: int) -> int:
        return self._lib.pt_batch_target_device_ptr(self._h, target) or 0

    def rmse(self, target: int, reference: int) -> float:
        out = ctypes.c_double()
        self._check(self._lib.pt_batch_rmse(self._h, target, reference, ctypes.byref(out)))
        return out.value

    def rmse_many(self, targets: list[int], references: list[int]) -> list[float]:
        n = len(targets)
        t = (ctypes.c_int * max(1, n))(*targets)
        r = (ctypes.c_int * max(1, n))(*references)
        out = (ctypes.c_double * max(1, n))()
        self._check(self._lib.pt_batch_rmse_many(self._h, t, r, n, out))
        return list(out[:n])

    def rmse_image(self, d_image: int, width: int, height: int, reference: int) -> float:
        out = ctypes.c_double()
        self._check(self._lib.pt_batch_rmse_image(self._h, d_image, width, height, reference, ctypes.byref(out)))
        return out.value

    def release_target(self, target: int):
        self._check(self._lib.pt_batch_release_target(self._h, target))

    def release_scene(self, scene: int):
        self._check(self._lib.pt_batch_release_scene(self._h, scene))


class Server:
    """pt_server: progressive render serving with error targets (libpt_host)."""

    def __init__(self, device: int = 0, mode: int = native.PT_SERVE_BATCHED, spp_per_pass: int = 8,
                 hbm_budget: int = 64 << 30, pool_slots: int = 1 << 21, max_passes: int = 4096,
                 iterations_per_poll: int = 4, passes_in_flight: int = 1, keep_images: bool = False,
                 fp64_paths: bool = False):
        self._lib = native.host()
        opts = native.PtServerOpts(mode, spp_per_pass, hbm_budget, pool_slots, max_passes, iterations_per_poll,
                                   passes_in_flight, int(keep_images), int(fp64_paths))
        h = ctypes.c_void_p()
        rc = self._lib.pt_server_create(ctypes.byref(h), device, ctypes.byref(opts))
        if rc != native.PT_OK:
            raise PathTracerError(rc, "pt_server_create failed")
        self._h = h
        self._sizes: dict[int, tuple[int, int]] = {}

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.pt_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    def _check(self, rc: int):
        if rc != native.PT_OK:
            raise PathTracerError(rc, self._lib.pt_server_last_error(self._h).decode())

    def now(self) -> float:
        return self._lib.pt_server_now(self._h)

    def set_mode(self, mode: int):
        self._check(self._lib.pt_server_set_mode(self._h, mode))

    def add_scene(self, key: int, ubo: np.ndarray, plugins: list):
        ubo = np.ascontiguousarray(ubo, np.float32)
        arr = (native.PtSdfPlugin * max(1, len(plugins)))(*plugins)
        self._check(self._lib.pt_server_add_scene(self._h, key, native.ptr(ubo), arr, len(plugins)))

    def add_scene_sources(self, key: int, ubo: np.ndarray, sources: list[str]):
        ubo = np.ascontiguousarray(ubo, np.float32)
        arr = (ctypes.c_char_p * max(1, len(sources)))(*[t.encode() for t in sources])
        self._check(self._lib.pt_server_add_scene_sources(self._h, key, native.ptr(ubo), arr, len(sources)))

    def set_scene_ext(self, key: int, ext):
        """pt_server_set_scene_ext (ext None: the reference's method)."""
        self._check(self._lib.pt_server_set_scene_ext(self._h, key, ctypes.byref(ext) if ext is not None else None))

    def render_reference(self, key: int, push: PtPush, spp: int, spp_per_pass: int = 32):
        self._check(self._lib.pt_server_render_reference(self._h, key, ctypes.byref(push), spp, spp_per_pass))

    @staticmethod
    def job(scene_key: int, push: PtPush, max_spp: int, target_rmse: float = 0.0) -> native.PtServerJob:
        return native.PtServerJob(scene_key, max_spp, target_rmse, push)

    def submit(self, job: native.PtServerJob) -> int:
        out = ctypes.c_uint64()
        self._check(self._lib.pt_server_submit(self._h, ctypes.byref(job), ctypes.byref(out)))
        self._sizes[out.value] = (job.push.resolution[0], job.push.resolution[1])
        return out.value

    def poll(self, capacity: int = 256) -> list[native.PtServerResult]:
        buf = (native.PtServerResult * capacity)()
        n = ctypes.c_int()
        self._check(self._lib.pt_server_poll(self._h, buf, capacity, ctypes.byref(n)))
        return [buf[i] for i in range(n.value)]

    def pending(self) -> int:
        return self._lib.pt_server_pending(self._h)

    def drain(self) -> list[native.PtServerResult]:
        out = []
        while self.pending() > 0:
            out += self.poll()
        return out

    def read_image(self, job_id: int) -> np.ndarray:
        w, h = self._sizes[job_id]
        out = np.empty((h, w, 4), np.float32)
        self._check(self._lib.pt_server_read_image(self._h, ctypes.c_uint64(job_id), native.ptr(out), out.nbytes))
        return out

    def release(self, job_id: int):
        self._check(self._lib.pt_server_release(self._h, ctypes.c_uint64(job_id)))

    def cancel(self, job_id: int):
        self._check(self._lib.pt_server_cancel(self._h, ctypes.c_uint64(job_id)))

    def stats(self) -> dict:
        st = native.PtServerStats()
        self._check(self._lib.pt_server_get_stats(self._h, ctypes.byref(st)))
        return {k: getattr(st, k) for k, _ in native.PtServerStats._fields_}

    def run_trace(self, jobs: list, arrivals: list[float]) -> list[native.PtServerResult]:
        n = len(jobs)
        arr_j = (native.PtServerJob * max(1, n))(*jobs)
        arr_t = (ctypes.c_double * max(1, n))(*arrivals)
        res = (native.PtServerResult * max(1, n))()
        self._check(self._lib.pt_server_run_trace(self._h, arr_j, arr_t, n, res))
        return [res[i] for i in range(n)]


def render_offscreen(ctx: Context, scene: Scene, cie: np.ndarray, width: int, height: int, num_samples: int,
                     spf: int, path_length: int, shot: int = 1, tonemap: int = 3, frame_offset: int = 0):
    """The reference's offscreen render; returns (accumulator HxWx4, seconds)."""
    cie = np.ascontiguousarray(cie, np.float32)
    opts = PtOffscreenOpts(width, height, num_samples, spf, path_length, shot, tonemap, frame_offset)
    out = np.empty((height, width, 4), np.float32)
    secs = ctypes.c_double()
    rc = native.host().pt_render_offscreen(ctx.handle, scene.handle, native.ptr(cie), ctypes.byref(opts),
                                           native.ptr(out), out.nbytes, ctypes.byref(secs))
    if rc != native.PT_OK:
        raise PathTracerError(rc, native.cuda().pt_last_error(ctx.handle).decode())
    ctx.width, ctx.height = width, height
    return out, secs.value


def export_rgb8(accum: np.ndarray, tonemap: int = 3) -> np.ndarray:
    """SaveRender's tonemap chain on the host: HxWx4 float -> HxWx3 uint8."""
    accum = np.ascontiguousarray(accum, np.float32)
    h, w = accum.shape[:2]
    rgb = np.empty((h, w, 3), np.uint8)
    rc = native.host().pt_export_rgb8(native.ptr(accum), w, h, tonemap, native.ptr(rgb))
    if rc != native.PT_OK:
        raise PathTracerError(rc, "export failed")
    return rgb


def glsl_translate(glsl: str, prefix: str = "u0_") -> str:
    """An SDF snippet's GLSL as the C++ the run-time compiled megakernel
    includes (functions renamed <prefix><name>); raises on unsupported text."""
    lib = native.cuda()
    need = ctypes.c_size_t()
    err = ctypes.create_string_buffer(256)
    rc = lib.pt_glsl_translate(glsl.encode(), prefix.encode(), None, 0, ctypes.byref(need), err, len(err))
    if rc != native.PT_OK:
        raise PathTracerError(rc, err.value.decode())
    out = ctypes.create_string_buffer(need.value)
    rc = lib.pt_glsl_translate(glsl.encode(), prefix.encode(), out, need.value, ctypes.byref(need), err, len(err))
    if rc != native.PT_OK:
        raise PathTracerError(rc, err.value.decode())
    return out.value.decode()


def jit_check(sources: list[str], sm: int = 103) -> str:
    """Compiles the run-time kernels a context builds for these snippets
    (pt_jit_check) without a GPU; returns the compiler log, raises with it
    on failure."""
    arr = (ctypes.c_char_p * max(1, len(sources)))(*[s.encode() for s in sources])
    log = ctypes.create_string_buffer(1 << 16)
    rc = native.cuda().pt_jit_check(arr, len(sources), sm, log, len(log))
    if rc != native.PT_OK:
        raise PathTracerError(rc, log.value.decode())
    return log.value.decode()
