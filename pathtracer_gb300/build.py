"""Builds the native libraries in-tree: libpt_cuda.so (nvcc, sm_103a) and
libpt_host.so (g++), into pathtracer_gb300/lib/.

No cmake: each library is one compiler invocation, and the independent ones
run in parallel.  Kernels are compiled with -fmad=false (every a*b+c stays
two roundings, as the shader's expressions are written; fma only where the
shader says fma) and IEEE division and square root (nvcc's defaults).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "lib")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
NVCC_FLAGS = [ARCH, "-O3", "-lineinfo", "-fmad=false", "-std=c++17", "-Xcompiler", "-fPIC,-Wall"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", "-Wextra"]

CUDA_SOURCES = [
    "kernel/pt_megakernel.cu",
    "kernel/pt_megakernel_analytic.cu",
    "kernel/pt_fp64.cu",
    "kernel/pt_wavefront.cu",
    "kernel/pt_wavefront_checked.cu",
    "pt_api.cu",
    "pt_engine.cu",
    "pt_noalloc.cu",
    "pt_batch.cu",
    "pt_export.cu",
    "pt_sdf_source.cpp",
    "pt_glsl.cpp",
    "pt_jit.cu",
]
# Headers the run-time compiled megakernel (pt_jit.cu) includes, under the
# names their #include lines use; embedded into libpt_cuda as strings.
JIT_HEADERS = [
    ("../../../include/pt_cuda.h", "include/pt_cuda.h"),
    ("../../../include/pt_mathf.h", "include/pt_mathf.h"),
    ("pt_vec.cuh", "pathtracer_gb300/csrc/kernel/pt_vec.cuh"),
    ("pt_scene.cuh", "pathtracer_gb300/csrc/kernel/pt_scene.cuh"),
    ("pt_features.h", "pathtracer_gb300/csrc/kernel/pt_features.h"),
    ("pt_geometry.cuh", "pathtracer_gb300/csrc/kernel/pt_geometry.cuh"),
    ("pt_path.cuh", "pathtracer_gb300/csrc/kernel/pt_path.cuh"),
    ("pt_megakernel.h", "pathtracer_gb300/csrc/kernel/pt_megakernel.h"),
    ("pt_megakernel_body.cuh", "pathtracer_gb300/csrc/kernel/pt_megakernel_body.cuh"),
    ("pt_wavefront.h", "pathtracer_gb300/csrc/kernel/pt_wavefront.h"),
    ("pt_march.cuh", "pathtracer_gb300/csrc/kernel/pt_march.cuh"),
    ("pt_glsl_shim.h", "pathtracer_gb300/csrc/kernel/pt_glsl_shim.h"),
]
GEN = os.path.join(LIB, "gen")
HOST_SOURCES = [
    "host/pt_json.cpp",
    "host/pt_scene.cpp",
    "host/pt_offscreen.cpp",
    "host/pt_generate.cpp",
    "host/pt_server.cpp",
]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libpt_cuda needs the CUDA toolkit")


def _cuda_home(nvcc: str) -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}")


def _stale(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    deps = list(sources)
    for d in (os.path.join(CSRC, "kernel"), os.path.join(CSRC, "host"), os.path.join(ROOT, "include")):
        deps += [os.path.join(d, f) for f in os.listdir(d)]
    return any(os.path.getmtime(s) > t for s in deps if os.path.isfile(s))


def _write_jit_sources() -> None:
    """pt_jit_sources.inc: the JIT_HEADERS texts as C++ raw string literals."""
    os.makedirs(GEN, exist_ok=True)
    names, texts = [], []
    for name, rel in JIT_HEADERS:
        with open(os.path.join(ROOT, rel)) as f:
            text = f.read()
        if ")PTSRC\"" in text:
            raise RuntimeError(f"{rel} contains the raw-string delimiter")
        names.append(f'"{name}"')
        texts.append('R"PTSRC(' + text + ')PTSRC"')
    body = ("// Generated by pathtracer_gb300/build.py from the kernel headers.\n"
            f"static const int kJitHeaderCount = {len(names)};\n"
            "static const char* const kJitHeaderNames[] = {" + ", ".join(names) + "};\n"
            "static const char* const kJitHeaderTexts[] = {\n" + ",\n".join(texts) + "};\n")
    out = os.path.join(GEN, "pt_jit_sources.inc")
    if not os.path.exists(out) or open(out).read() != body:
        with open(out, "w") as f:
            f.write(body)


def build(force: bool = False, verbose: bool = False) -> dict[str, str]:
    """Compiles both libraries (if stale) and returns their paths."""
    os.makedirs(LIB, exist_ok=True)
    nvcc = _nvcc()
    cuda_inc = os.path.join(_cuda_home(nvcc), "include")
    cuda_so = os.path.join(LIB, "libpt_cuda.so")
    host_so = os.path.join(LIB, "libpt_host.so")
    cuda_src = [os.path.join(CSRC, s) for s in CUDA_SOURCES]
    host_src = [os.path.join(CSRC, s) for s in HOST_SOURCES]

    host_cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, f"-I{cuda_inc}", "-o", host_so, *host_src,
                f"-L{LIB}", "-lpt_cuda", "-Wl,-rpath,$ORIGIN"]

    _write_jit_sources()
    if force or _stale(cuda_so, cuda_src + [os.path.join(GEN, "pt_jit_sources.inc")]):
        # One object per translation unit, compiled in parallel, then linked.
        objdir = os.path.join(LIB, "obj")
        os.makedirs(objdir, exist_ok=True)
        objs = [os.path.join(objdir, os.path.basename(s) + ".o") for s in cuda_src]
        cmds = [[nvcc, *NVCC_FLAGS, f"-I{GEN}", "-c", "-o", o, s] for s, o in zip(cuda_src, objs)]
        if verbose:
            for c in cmds:
                print(" ".join(c), file=sys.stderr)
        with ThreadPoolExecutor(max_workers=min(len(cmds), os.cpu_count() or 1)) as ex:
            list(ex.map(_run, cmds))
        link = [nvcc, ARCH, "-shared", "-o", cuda_so, *objs, "-lnvrtc"]
        if verbose:
            print(" ".join(link), file=sys.stderr)
        _run(link)
    if force or _stale(host_so, host_src) or os.path.getmtime(cuda_so) > os.path.getmtime(host_so):
        if verbose:
            print(" ".join(host_cmd), file=sys.stderr)
        _run(host_cmd)
    return {"cuda": cuda_so, "host": host_so}


def build_oracle(force: bool = False) -> str:
    """Compiles the oracle (oracle/: the CPU restatement the tests check against)."""
    out = os.path.join(ROOT, "oracle", "_build", "libpt_oracle.so")
    src = os.path.join(ROOT, "oracle", "pt_oracle.c")
    hdrs = [os.path.join(ROOT, "oracle", "pt_oracle.h"), os.path.join(ROOT, "include", "pt_cuda.h"),
            os.path.join(ROOT, "include", "pt_mathf.h")]
    if force or not os.path.exists(out) or any(os.path.getmtime(s) > os.path.getmtime(out) for s in [src, *hdrs]):
        os.makedirs(os.path.dirname(out), exist_ok=True)
        _run([os.environ.get("CC", "gcc"), "-O2", "-fPIC", "-std=c11", "-ffp-contract=off", "-fno-fast-math",
              "-fopenmp", "-shared", "-o", out, src, "-lm"])
    return out


def build_all(force: bool = False) -> dict[str, str]:
    with ThreadPoolExecutor(max_workers=2) as ex:
        fo = ex.submit(build_oracle, force)
        fl = ex.submit(build, force)
        paths = fl.result()
        paths["oracle"] = fo.result()
    return paths


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
