"""CPU baselines of the five workloads, timed on the oracle.

Measurement infrastructure, like the rest of oracle/: only bench.py's CPU
baseline leg and its reference arm import this module.  Each function times
the oracle (the C++ restatement of pixie's scalar path, oracle/pxo.cpp) on a
bounded sample of one workload, one thread, and returns seconds plus the
units processed.  ``all_cores`` runs the same sample in one spawned process
per core (independent jobs, as a caller of the single-threaded reference
would run them) and returns the aggregate rate.
"""
from __future__ import annotations

import multiprocessing as mp
import os
import platform
import sys
import time

_ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _imports():
    if _ROOT not in sys.path:
        sys.path.insert(0, _ROOT)
    from oracle import pxo
    from pixie_gb300 import workloads as wl
    return pxo, wl


def host() -> dict:
    return {"uname_m": platform.machine(), "nproc": os.cpu_count()}


def plain_fill(n_paths: int = 40) -> tuple[float, int]:
    """512x512, one path of 64 random cubics per call (NonZero, Normal,
    opaque pink), n_paths calls drawn over one image as the GPU leg does."""
    pxo, wl = _imports()
    img = pxo.new_image(512, 512)
    paths = [wl.plain_path(s) for s in range(1, n_paths + 1)]
    t = time.perf_counter()
    for c in paths:
        pxo.fill_path(img, c, wl.PLAIN_COLOR)
    return time.perf_counter() - t, n_paths


def dense_scene(n_paths: int = 150, seed: int = 7) -> tuple[float, int]:
    """The first n_paths of the 2000-path dense scene on its 1024x1024 canvas,
    drawn in order (paths the reference raises for are skipped)."""
    pxo, wl = _imports()
    items = wl.dense_scene(seed, n_paths=2000, size=1024.0)[:n_paths]
    img = pxo.new_image(1024, 1024)
    t = time.perf_counter()
    pxo.draw_items(img, items, 1)
    return time.perf_counter() - t, n_paths


def glyphs(n: int = 512, seed: int = 7) -> tuple[float, int]:
    """One fillPath per glyph into its own image, then one draw per glyph onto
    a 4096x4096 page, for the first n glyphs of the 4096-glyph batch."""
    pxo, wl = _imports()
    gl, pos = wl.glyph_batch(seed, n=4096, page=4096)
    page = pxo.new_image(4096, 4096)
    t = time.perf_counter()
    for (cmds, w, h, wind), (x, y) in zip(gl[:n], pos[:n]):
        m = pxo.new_image(w, h)
        pxo.fill_path(m, cmds, [1, 1, 1, 1], 1.0, 0, None, wind)
        pxo.draw(page, m, int(x), int(y), 0)
    return time.perf_counter() - t, n


def serving_job(seed: int, paths: int = 60) -> tuple[float, int]:
    """The first `paths` paths of one serving job (canvas side log-U[256, 4096]),
    plus its blur when it has one; returns (seconds, the job's path count) so
    the caller can scale the time per path to the whole job."""
    pxo, wl = _imports()
    job = wl.serving_job(seed)
    img = pxo.new_image(job["side"], job["side"])
    t = time.perf_counter()
    pxo.draw_items(img, job["items"][:paths], 1)
    dt = time.perf_counter() - t
    n = len(job["items"])
    dt *= n / max(1, min(paths, n))
    if job["blur"]:
        t = time.perf_counter()
        pxo.blur(img, job["blur"])
        dt += time.perf_counter() - t
    return dt, 1


SAMPLES = {"plain_fill": plain_fill, "dense_scene": dense_scene, "glyphs": glyphs, "serving_job": serving_job}


def _worker(args):
    name, kw = args
    return SAMPLES[name](**kw)


def all_cores(name: str, kw_per_core: list[dict]) -> tuple[float, int, float]:
    """Runs SAMPLES[name] once per core in spawned processes (the oracle holds
    no GPU state; spawn keeps the pool independent of any CUDA context).
    Returns (wall seconds, units in all, summed single-process seconds)."""
    ctx = mp.get_context("spawn")
    with ctx.Pool(len(kw_per_core)) as pool:
        pool.map(_worker, [(name, kw_per_core[0])] * len(kw_per_core))  # warm: imports, library load
        t = time.perf_counter()
        res = pool.map(_worker, [(name, kw) for kw in kw_per_core])
        wall = time.perf_counter() - t
    return wall, sum(r[1] for r in res), sum(r[0] for r in res)
