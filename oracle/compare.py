"""Per-sample comparison of libpt_cuda against the CPU restatement.

TEST INFRASTRUCTURE ONLY (tests, smoke check, bench CPU baseline).

Parity definition: for every path (pixel, sample) both sides record the
branch sequence of each bounce — hit object / SDF / miss, emitter hit, light
picked, shadow-ray outcome, Russian-roulette kill — plus the sample's XYZ.
A path "matches" when its whole sequence is identical.  Required: at least
99.9% of paths match; matching paths agree in XYZ within 1e-4 relative; and
pixels whose paths all match agree in accumulated XYZ within 1e-4 relative.
Transcendentals (sin, cos, exp, log, pow, acos) come from different
libraries on the two sides (glibc vs CUDA), so rare one-ulp differences can
flip a comparison and send a path another way; that is what the 0.1% allows.
"""
from __future__ import annotations

import ctypes

import numpy as np

from pathtracer_gb300 import native

from . import oracle

REL_TOL = 1e-4
PATH_MATCH_MIN = 0.999


def plugins_for(scene, custom: dict | None = None) -> list:
    """The oracle's plug-in per SDF of the scene.  Text that is not one of the
    shipped snippets is registered for its slot as PT_SDF_CUSTOM with its C
    restatement in user_sdfs.c: from `custom` (source text -> the names of
    its sdf and material functions) or, for the texts of the repository's
    scenes and generator, oracle.restatement_for."""
    out = []
    for slot, src in enumerate(scene.sdf_sources()):
        p = native.PtSdfPlugin()
        rc = native.cuda().pt_parse_sdf_source(src.encode(), ctypes.byref(p))
        if rc != native.PT_OK:
            names = custom[src] if custom and src in custom else oracle.restatement_for(src)
            if names is None:
                raise ValueError(f"unsupported SDF source: {src[:60]!r}")
            oracle.set_user_sdf(slot, *names)
            p = native.plugin(native.PT_SDF_CUSTOM)
        out.append(p)
    return out


def run_oracle(ubo, push, plugins, accum=None, rect=None, trace_depth=0, nthreads=0, ext=None):
    W, H = push.resolution[0], push.resolution[1]
    if accum is None:
        accum = np.zeros((H, W, 4), np.float32)
    tr = oracle.dispatch(ubo, push, plugins, accum, rect=rect, trace_depth=trace_depth, nthreads=nthreads, ext=ext)
    return accum, tr


def run_gpu(ctx, push, trace_depth=0):
    """One pt_dispatch with optional per-path trace (torch CUDA buffers)."""
    import torch

    W, H = push.resolution[0], push.resolution[1]
    spf = push.samplesPerFrame
    tr = None
    if trace_depth > 0:
        npaths = W * H * spf
        ev = torch.zeros(npaths * trace_depth, dtype=torch.int32, device="cuda")
        nev = torch.zeros(npaths, dtype=torch.int32, device="cuda")
        col = torch.zeros(npaths * 3, dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        ctx.set_trace(ev.data_ptr(), nev.data_ptr(), col.data_ptr(), trace_depth)
        tr = (ev, nev, col)
    ctx.dispatch(push)
    ctx.wait()
    if tr is not None:
        ctx.set_trace(0, 0, 0, 0)
        ev, nev, col = tr
        npaths = W * H * spf
        tr = (ev.cpu().numpy().view(np.uint32).reshape(npaths, trace_depth), nev.cpu().numpy().view(np.uint32),
              col.cpu().numpy().reshape(npaths, 3))
    return ctx.read_accum(), tr


def _rel(a, b, floor):
    return np.abs(a - b) / np.maximum(np.maximum(np.abs(a), np.abs(b)), floor)


def compare(acc_o, tr_o, acc_g, tr_g, spf, rect=None, W=None):
    """Returns a report dict; tr_* = (events[npaths, depth], nevents[npaths], colors[npaths, 3]).

    With rect=(x0, y0, x1, y1) the oracle covered only that rectangle and the
    GPU arrays (full frame) are cut to it."""
    ev_o, nev_o, col_o = tr_o
    ev_g, nev_g, col_g = tr_g
    if rect is not None:
        x0, y0, x1, y1 = rect
        Hf = acc_g.shape[0]
        Wf = acc_g.shape[1]
        depth = ev_g.shape[1]
        ev_g = ev_g.reshape(Hf, Wf, spf, depth)[y0:y1, x0:x1].reshape(-1, depth)
        nev_g = nev_g.reshape(Hf, Wf, spf)[y0:y1, x0:x1].reshape(-1)
        col_g = col_g.reshape(Hf, Wf, spf, 3)[y0:y1, x0:x1].reshape(-1, 3)
        acc_g = acc_g[y0:y1, x0:x1]
        acc_o = acc_o[y0:y1, x0:x1]
    depth = ev_o.shape[1]
    cap = np.minimum(nev_o, depth)
    mask = np.arange(depth)[None, :] < cap[:, None]
    same_ev = np.all(np.where(mask, ev_o == ev_g, True), axis=1)
    path_ok = same_ev & (nev_o == nev_g)
    npaths = path_ok.size
    path_frac = float(path_ok.mean()) if npaths else 1.0
    floor_c = max(1e-6, float(np.abs(col_o).max()) * 1e-6) if npaths else 1e-6
    rel_c = _rel(col_o, col_g, floor_c).max(axis=1) if npaths else np.zeros(0)
    color_bad = int(np.count_nonzero(rel_c[path_ok] > REL_TOL)) if npaths else 0
    pix_ok = path_ok.reshape(-1, spf).all(axis=1)
    xo = acc_o[..., :3].reshape(-1, 3)
    xg = acc_g[..., :3].reshape(-1, 3)
    floor_p = max(1e-6, float(np.abs(xo).max()) * 1e-6)
    rel_p = _rel(xo, xg, floor_p).max(axis=1)
    pix_bad = int(np.count_nonzero(rel_p[pix_ok] > REL_TOL))
    return {
        "paths": npaths,
        "path_match": path_frac,
        "color_max_rel_matched": float(rel_c[path_ok].max()) if path_ok.any() else 0.0,
        "color_bad": color_bad,
        "pixels": int(pix_ok.size),
        "pixels_all_match": float(pix_ok.mean()),
        "pixel_max_rel_matched": float(rel_p[pix_ok].max()) if pix_ok.any() else 0.0,
        "pixel_bad": pix_bad,
        "w_ok": bool(np.all(acc_g[..., 3] == 1.0)),
    }


def passes(report) -> bool:
    return (report["path_match"] >= PATH_MATCH_MIN and report["color_bad"] == 0 and report["pixel_bad"] == 0
            and report["w_ok"])
