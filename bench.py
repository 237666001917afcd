#!/usr/bin/env python3
"""Benchmark of pixie's raster hot path on GB300 (one JSON line on stdout).

Workload (the composite-and-blur configuration): per step
  * draw() of a 2048x2048 premultiplied RGBX image onto another under each of
    the 16 blend modes and the 4 mask modes (20 destination/source pairs, so
    a step's working set, 640 MB, is far larger than the 129 MB L2);
  * gaussian blur of a 4096x4096 image at radius 1, 4, 16 and 64;
  * shadow (offset (8, 8), spread 4, blur 12) of a 1024x1024 mask of 64 discs.
Metric unit: Gpix/s = pixels processed (20 x 2048^2 + 4 x 4096^2 + 1024^2)
per step / step time.  Inputs are seeded synthetic data with the shapes and
value distributions of the configuration.

  --impl pxg        (default) the CUDA library through its C ABI
  --impl reference  the reference's CPU path (the C++ restatement in oracle/,
                    pixie itself is Nim and cannot be built here) on all host
                    cores, on a bounded sample of the same workload
Also reported: the plain per-call fillPath (512x512, 64 random cubics) and
the batched 4096-glyph fill, in "extra".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "paths/s & Gpix/s on 1 GB300, batched vs plain GPU, bit-exact; p50/p99 job latency"
DRAW_W = 2048
BLUR_W = 4096
RADII = (1, 4, 16, 64)
SHADOW_W = 1024
N_MODES = 20
STEP_PIXELS = N_MODES * DRAW_W * DRAW_W + len(RADII) * BLUR_W * BLUR_W + SHADOW_W * SHADOW_W
WORKLOAD = {"workload": "composite+blur: draw 2048^2 x 20 modes, blur 4096^2 r in {1,4,16,64}, "
                        "shadow 1024^2 (offset 8,8 spread 4 blur 12)",
            "draw_images": "20 dst + 20 src 2048x2048 RGBX", "blur_image": "4096x4096 RGBX x 4",
            "l2": "inputs larger than L2: 640 MB of draw images cycled per step"}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# -- clocks -------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples every 100 ms while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        time.sleep(0.15)
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# -- distributed helpers ----------------------------------------------------------------
def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:  # host-only replicas (tests of the N>1 timing path)
            dist.init_process_group("gloo")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, v):
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# -- GPU arm ------------------------------------------------------------------------------
def run_gpu(args, ws, rank, local):
    import torch

    import pixie_gb300 as px
    from pixie_gb300 import workloads as wl

    torch.cuda.set_device(local)
    px.lib().pxg_init(local)
    stream = torch.cuda.Stream()
    px.set_stream(stream.cuda_stream)

    seed = 1 + rank
    a_host = [wl.premultiplied_image(seed * 10 + i, DRAW_W, DRAW_W) for i in range(2)]
    b_host = [wl.premultiplied_image(seed * 10 + 5 + i, DRAW_W, DRAW_W) for i in range(2)]
    blur_host = wl.premultiplied_image(seed * 10 + 9, BLUR_W, BLUR_W)
    A = [px.Image.from_numpy(a_host[i % 2]) for i in range(N_MODES)]
    B = [px.Image.from_numpy(b_host[i % 2]) for i in range(N_MODES)]
    BL = [px.Image.from_numpy(blur_host) for _ in RADII]
    M = px.Image(SHADOW_W, SHADOW_W)
    M.fill_path(wl.disc_mask_path(seed), [1, 1, 1, 1])
    SH = px.Image(SHADOW_W, SHADOW_W)
    black = [0, 0, 0, 1]
    px.set_blocking(False)

    ops = ([("draw", k) for k in range(N_MODES)] + [("blur", r) for r in RADII] + [("shadow", 0)])

    def run_op(op):
        kind, p = op
        if kind == "draw":
            A[p].draw(B[p], (0, 0), p)
        elif kind == "blur":
            BL[RADII.index(p)].blur(p)
        else:
            M.shadow_into(SH, (8, 8), 4, 12, black)

    # warm-up; its last step is instrumented to find the dominant operation
    n_ops = len(ops)
    wev = [torch.cuda.Event(enable_timing=True) for _ in range(n_ops + 1)]
    with torch.cuda.stream(stream):
        for w in range(args.warmup):
            for i, op in enumerate(ops):
                if w == args.warmup - 1:
                    wev[i].record(stream)
                run_op(op)
            if w == args.warmup - 1:
                wev[n_ops].record(stream)
    stream.synchronize()
    dom = int(np.argmax([wev[i].elapsed_time(wev[i + 1]) for i in range(n_ops)])) if args.warmup else 0

    # timed region: K steps bracketed by two events on the library's stream;
    # the dominant operation alone is bracketed by events inside it (its
    # kernels' duration for the roofline)
    dev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    l0 = px.launch_count()
    barrier(ws)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        h0 = time.perf_counter()
        for s in range(args.steps):
            for i, op in enumerate(ops):
                if i == dom:
                    dev[s][0].record(stream)
                    run_op(op)
                    dev[s][1].record(stream)
                else:
                    run_op(op)
        t1.record(stream)
        host_ms = (time.perf_counter() - h0) * 1e3 / args.steps  # enqueue time per step on the host
        stream.synchronize()
        torch.cuda.synchronize()
        barrier(ws)
    launches = (px.launch_count() - l0) // args.steps
    total_ms = max_over_ranks(ws, t0.elapsed_time(t1))
    ms_step = total_ms / args.steps

    # per-operation breakdown, outside the timed region: events around every op
    # over a few more steps (the events add small gaps between operations)
    n_prof = max(1, min(args.steps, 5))
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(n_ops + 1)] for _ in range(n_prof)]
    for s in range(n_prof):
        for i, op in enumerate(ops):
            evs[s][i].record(stream)
            run_op(op)
        evs[s][n_ops].record(stream)
    stream.synchronize()
    op_ms = np.zeros(n_ops)
    for s in range(n_prof):
        for i in range(n_ops):
            op_ms[i] += evs[s][i].elapsed_time(evs[s][i + 1])
    op_ms /= n_prof

    # roofline of the dominant operation, timed inside the timed region
    dom_ms = float(np.mean([a.elapsed_time(b) for a, b in dev]))
    kind, p = ops[dom]
    if kind == "draw":
        bpp = 8 if p == 17 else 12
        algo = bpp * DRAW_W * DRAW_W
        unit_desc = f"draw mode {p}: {bpp} B/px x 2048^2 px"
    elif kind == "blur":
        algo = 8 * BLUR_W * BLUR_W
        unit_desc = f"blur r={p}: 8 B/px x 4096^2 px (X and Y pass, read once + write once)"
    else:
        algo = 5 * SHADOW_W * SHADOW_W
        unit_desc = "shadow: 5 B/px x 1024^2 px"
    peak, peak_src = peaks()
    achieved = algo / (dom_ms * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": f"{kind}:{p}", "unit_bytes": algo, "unit": "GB/s",
            "achieved": round(achieved, 1), "peak": peak, "peak_source": peak_src,
            "frac": round(achieved / peak, 4), "traffic": TRAFFIC.get(f"{kind}:{p}"),
            "per_launch": unit_desc}
    draw_ms = op_ms[:N_MODES]
    draw_gbs = [(8 if m == 17 else 12) * DRAW_W * DRAW_W / (t * 1e-3) / 1e9 for m, t in enumerate(draw_ms)]
    blur_ms = {r: round(float(op_ms[N_MODES + i]), 4) for i, r in enumerate(RADII)}

    # end to end through the C ABI with host buffers (pinned), copies timed
    e2e = run_e2e(px, A, B, BL, M, SH, a_host, b_host, blur_host, run_op, ops, args, ws)

    extra = {"per_op_ms": {f"{k}:{p}": round(float(t), 4) for (k, p), t in zip(ops, op_ms)},
             "host_enqueue_ms_per_step": round(host_ms, 4),
             "draw_gbs_min_median_max": [round(min(draw_gbs), 1), round(statistics.median(draw_gbs), 1),
                                         round(max(draw_gbs), 1)],
             "blur_ms": blur_ms}
    parity = None
    if rank == 0 and not args.no_parity:
        parity = check_parity(px, A, B, BL, M, SH, a_host, b_host, blur_host, seed)
    if rank == 0 and not args.no_fill:
        extra.update(run_fill_extras(px, wl, args, stream))
    return ms_step, launches, roof, e2e, extra, clk.summary(), parity


def check_parity(px, A, B, BL, M, SH, a_host, b_host, blur_host, seed):
    """Outside the timed region: every operation of the step once more on
    fresh copies of its seeded inputs, compared byte for byte with the
    oracle's render of the same inputs (the oracle's calls run in threads)."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle import pxo
    from pixie_gb300 import workloads as wl
    pxo.set_golden_mode(False)

    def ref_draw(mode):
        r = a_host[mode % 2].copy()
        pxo.draw(r, b_host[mode % 2], 0, 0, mode)
        return r

    def ref_blur(r):
        x = blur_host.copy()
        pxo.blur(x, r)
        return x

    def ref_shadow():
        m = pxo.new_image(SHADOW_W, SHADOW_W)
        pxo.fill_path(m, wl.disc_mask_path(seed), [1, 1, 1, 1])
        return pxo.shadow(m, 8, 8, 4, 12, [0, 0, 0, 1])

    t = time.perf_counter()
    with ThreadPoolExecutor(min(16, os.cpu_count() or 1)) as ex:
        f_draw = {m: ex.submit(ref_draw, m) for m in range(N_MODES)}
        f_blur = {r: ex.submit(ref_blur, r) for r in RADII}
        f_sh = ex.submit(ref_shadow)
        got = {}
        for m in range(N_MODES):  # the GPU side meanwhile
            A[m].upload(a_host[m % 2])
            B[m].upload(b_host[m % 2])
            A[m].draw(B[m], (0, 0), m)
            got[f"draw:{m}"] = A[m].to_numpy()
        for i, r in enumerate(RADII):
            BL[i].upload(blur_host)
            BL[i].blur(r)
            got[f"blur:{r}"] = BL[i].to_numpy()
        M.shadow_into(SH, (8, 8), 4, 12, [0, 0, 0, 1])
        got["shadow:0"] = SH.to_numpy()
        want = {f"draw:{m}": f.result() for m, f in f_draw.items()}
        want.update({f"blur:{r}": f.result() for r, f in f_blur.items()})
        want["shadow:0"] = f_sh.result()
    worst, differing, bad = 0, 0, {}
    for k, g in got.items():
        d = np.abs(g.astype(np.int16) - want[k].astype(np.int16))
        mx, n = int(d.max()), int((d.reshape(-1, 4).max(axis=1) > 0).sum())
        worst, differing = max(worst, mx), differing + n
        if n:
            bad[k] = {"max_abs_delta": mx, "differing_px": n}
    return {"max_abs_delta": worst, "differing_px": differing, "ops_checked": len(got),
            "against": "oracle (scalar restatement of pixie), same seeded inputs, one fresh run of each "
                       "operation of the step at full size", "failing_ops": bad,
            "oracle_s": round(time.perf_counter() - t, 1)}


def run_e2e(px, A, B, BL, M, SH, a_host, b_host, blur_host, run_op, ops, args, ws):
    import torch
    pinned_a = [torch.from_numpy(a).pin_memory().numpy() for a in a_host]
    pinned_b = [torch.from_numpy(b).pin_memory().numpy() for b in b_host]
    pinned_blur = torch.from_numpy(blur_host).pin_memory().numpy()
    out_draw = torch.empty((DRAW_W, DRAW_W, 4), dtype=torch.uint8).pin_memory().numpy()
    out_blur = torch.empty((BLUR_W, BLUR_W, 4), dtype=torch.uint8).pin_memory().numpy()
    out_sh = torch.empty((SHADOW_W, SHADOW_W, 4), dtype=torch.uint8).pin_memory().numpy()
    mask_host = M.to_numpy()
    pinned_mask = torch.from_numpy(mask_host).pin_memory().numpy()
    steps = max(1, min(args.steps, args.e2e_steps))
    h2d = d2h = 0
    for warm in (True, False):  # one untimed step, then the timed ones
        barrier(ws)
        px.synchronize()
        t0 = time.perf_counter()
        for _ in range(1 if warm else steps):
            h2d = d2h = 0
            for k in range(N_MODES):  # inputs host -> device
                A[k].upload(pinned_a[k % 2])
                B[k].upload(pinned_b[k % 2])
                h2d += 2 * DRAW_W * DRAW_W * 4
            for im in BL:
                im.upload(pinned_blur)
                h2d += BLUR_W * BLUR_W * 4
            M.upload(pinned_mask)
            h2d += SHADOW_W * SHADOW_W * 4
            for op in ops:
                run_op(op)
            for k in range(N_MODES):  # results device -> host
                px.lib().pxg_image_download(A[k]._h, px._ptr(out_draw), out_draw.nbytes)
                d2h += out_draw.nbytes
            for im in BL:
                px.lib().pxg_image_download(im._h, px._ptr(out_blur), out_blur.nbytes)
                d2h += out_blur.nbytes
            px.lib().pxg_image_download(SH._h, px._ptr(out_sh), out_sh.nbytes)
            d2h += out_sh.nbytes
        px.synchronize()
        dt = time.perf_counter() - t0
    dt = max_over_ranks(ws, dt)
    return {"value": round(STEP_PIXELS * steps * int(os.environ.get("WORLD_SIZE", "1")) / dt / 1e9, 3),
            "unit": "Gpix/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "steps": steps, "ms_per_step": round(dt / steps * 1e3, 3)}


def run_fill_extras(px, wl, args, stream):
    """Plain per-call fillPath and the batched glyph fill (paths/s)."""
    out = {}
    img = px.Image(512, 512)
    paths = [np.ascontiguousarray(wl.plain_path(s), np.float32) for s in range(1, 41)]
    px.set_blocking(True)
    for c in paths[:5]:
        img.fill_path(c, wl.PLAIN_COLOR)
    # the C ABI as a Nim caller binds it: arguments built once, one blocking call per path
    L = px.lib()
    col = np.ascontiguousarray(wl.PLAIN_COLOR, np.float32)
    colp = px._ptr(col)
    args_c = [(px._ptr(c), c.size) for c in paths]
    t = time.perf_counter()
    gpu_ms = 0.0
    n = 0
    for rep in range(5):
        for ptr, size in args_c:
            if L.pxg_image_fill_path(img._h, ptr, size, colp, 1.0, 0, None, 0) != 0:
                raise px.PixieError(L.pxg_take_error().decode())
            gpu_ms += L.pxg_last_gpu_ms()
            n += 1
    dt = time.perf_counter() - t
    # the same calls through the Python mirror (argument conversion per call)
    t = time.perf_counter()
    for c in paths:
        img.fill_path(c, wl.PLAIN_COLOR)
    dt_py = time.perf_counter() - t
    segs = 0
    for c in paths:  # flattened segments (edges) per path, from the library's counters
        img.fill_path(c, wl.PLAIN_COLOR)
        segs += px.last_fill_stats()["segments"]
    edges_per_path = segs / len(paths)
    out["plain_fill_512_64cubics"] = {"paths_per_s": round(n / dt, 1),
                                      "edges_per_s": round(n / dt * edges_per_path, 1),
                                      "edges_per_path": round(edges_per_path, 1),
                                      "gpu_ms_per_path": round(gpu_ms / n, 4),
                                      "paths_per_s_python_api": round(len(paths) / dt_py, 1),
                                      "note": "one blocking C-ABI call per path (arguments prepared once, as a "
                                              "native caller holds them), host pre-pass included"}
    cpu = not args.no_cpu_baseline
    out["draw_transform_2048"] = run_draw_transform(px, wl, stream, cpu=cpu)
    out["paints_2048"] = run_paints(px, wl, stream, cpu=cpu)
    out["glyph_batch"] = run_glyphs(px, wl, args.glyphs)
    out["dense_scene_1024_2000"] = run_scene(px, wl)
    out["svg_tiger_900"] = run_svg_tiger(px, cpu=cpu)
    if args.serve_jobs > 0:
        rates = tuple(float(r) for r in args.serve_rates.split(",") if r)
        out["serving"] = run_serving(px, wl, args.serve_jobs, args.serve_pool, rates=rates)
    if cpu:
        add_cpu_baselines(out)
    px.set_blocking(False)
    return out


def add_cpu_baselines(out):
    """The oracle (C++ restatement of pixie's scalar path) on bounded samples
    of the fill, scene, glyph and serving workloads: one thread, and one
    independent sample per host core in spawned processes."""
    from oracle import cpu_baselines as cb
    cores = os.cpu_count() or 1
    host = cb.host()

    def both(name, kw, per_core_kw=None):
        t1, n1 = cb.SAMPLES[name](**kw)
        wall, n_all, _ = cb.all_cores(name, per_core_kw or [kw] * cores)
        return t1, n1, wall, n_all

    t1, n1, wall, n_all = both("plain_fill", {"n_paths": 200})
    pf = out["plain_fill_512_64cubics"]
    pf["cpu_oracle"] = {"paths_per_s_1core": round(n1 / t1, 1), "paths_per_s_all_cores": round(n_all / wall, 1),
                        "edges_per_s_1core": round(n1 / t1 * pf["edges_per_path"], 1),
                        "cores": cores, **host, "sample": "200 plain paths per process"}
    pf["gpu_over_cpu_1core"] = round(pf["paths_per_s"] / (n1 / t1), 1)
    t1, n1, wall, n_all = both("dense_scene", {"n_paths": 150})
    sc = out["dense_scene_1024_2000"]
    per_path = t1 / n1
    sc["cpu_oracle"] = {"paths_per_s_1core": round(1 / per_path, 2), "paths_per_s_all_cores": round(n_all / wall, 1),
                        "ms_per_scene_1core_est": round(per_path * 2000 * 1e3, 0),
                        "edges_per_s_1core": round(sc["segments"] / sc["paths_recorded"] / per_path, 1),
                        "cores": cores, **host,
                        "sample": "the scene's first 150 paths on its 1024^2 canvas per process, scaled per path"}
    sc["gpu_over_cpu_1core"] = round(sc["paths_per_s_gpu"] * per_path, 1)
    t1, n1, wall, n_all = both("glyphs", {"n": 1024})
    gb = out["glyph_batch"]
    gb["cpu_oracle"] = {"paths_per_s_1core": round(n1 / t1, 1), "paths_per_s_all_cores": round(n_all / wall, 1),
                        "cores": cores, **host,
                        "sample": "fillPath of the first 1024 glyphs into their own images + draw onto a "
                                  "4096^2 page, per process"}
    gb["batched_gpu_over_cpu_1core"] = round(gb["batched_paths_per_s"] / (n1 / t1), 1)
    if "serving" in out:
        seeds = out["serving"]["pool_seeds"][:4]
        per_job = [cb.serving_job(sd, 60)[0] for sd in seeds]
        mean_job = sum(per_job) / len(per_job)
        out["serving"]["cpu_oracle"] = {
            "s_per_job_1core_est": round(mean_job, 2), "jobs_per_s_1core_est": round(1 / mean_job, 3),
            "jobs_per_s_all_cores_est": round(cores / mean_job, 2), "cores": cores, **host,
            "sample": "4 pool jobs: their first 60 paths drawn and scaled per path to the whole job, plus the "
                      "job's blur; all cores = cores / time per job (independent jobs, as the other "
                      "workloads' all-core samples measure)"}


SMOOTH_CASES = {  # name: (column-major Mat3 of translate * rotate * scale, what it exercises)
    "rotate30_scale1.1": ((30.0, 1.1, 1.1, 1024.0, -300.0), "drawSmooth only"),
    "rotate10_scale0.3": ((10.0, 0.3, 0.3, 500.25, 400.5), "one minifyBy2 pre-pass + drawSmooth"),
    "translate_0.5": ((0.0, 1.0, 1.0, 0.5, 0.5), "fractional translation: drawSmooth"),
}


def smooth_mat(angle, sx, sy, tx, ty):
    import math
    import numpy as np
    a = math.radians(angle)
    c, s = math.cos(a), math.sin(a)
    return [float(np.float32(v)) for v in (c * sx, s * sx, 0, -s * sy, c * sy, 0, tx, ty, 1)]


def run_draw_transform(px, wl, stream, cpu=True, reps=20):
    """draw(a, b, Mat3, NormalBlend) of a 2048^2 source onto a 2048^2 canvas
    (GPU ms per draw, CUDA events) beside the CPU baseline: the oracle on a
    512^2 sample, scaled per pixel."""
    import torch
    out = {}
    srcs = [px.Image.from_numpy(wl.premultiplied_image(40 + i, 2048, 2048)) for i in range(2)]
    dsts = [px.Image.from_numpy(wl.premultiplied_image(50 + i, 2048, 2048)) for i in range(8)]
    px.set_blocking(False)
    for name, (geo, what) in SMOOTH_CASES.items():
        m = smooth_mat(*geo)
        for i in range(3):
            dsts[i % 8].draw_transform(srcs[i % 2], m, 0)
        px.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(reps):
            dsts[i % 8].draw_transform(srcs[i % 2], m, 0)
        e1.record(stream)
        px.synchronize()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        out[name] = {"gpu_ms": round(ms, 4), "what": what,
                     "canvas_gpix_per_s": round(2048 * 2048 / ms / 1e6, 2)}
        if cpu:  # CPU baseline: the oracle, one thread, a 512^2 source onto a 512^2 canvas
            from oracle import pxo
            small = smooth_mat(geo[0], geo[1], geo[2], geo[3] / 4, geo[4] / 4)
            a = wl.premultiplied_image(60, 512, 512)
            b = wl.premultiplied_image(61, 512, 512)
            t = time.perf_counter()
            pxo.draw_transform(a, b, small, 0)
            out[name]["cpu_oracle_ms_scaled_to_2048"] = round((time.perf_counter() - t) * 1000 * 16, 1)
    px.set_blocking(True)
    return out


PAINT_STOPS = [((1.0, 0.0, 0.0, 1.0), 0.0), ((0.2, 0.6, 1.0, 0.75), 0.4), ((0.0, 0.0, 0.5, 0.15625), 1.0)]
PAINT_HANDLES = {3: [(0.0, 1024.0), (2048.0, 1024.0)], 4: [(1024.0, 1024.0), (2048.0, 1024.0), (1024.0, 2048.0)],
                 5: [(1024.0, 1024.0), (2048.0, 1024.0), (1024.0, 2048.0)]}


def run_paints(px, wl, stream, cpu=True, reps=10):
    """Gradient fills of a 2048^2 image (fill(image, paint)) and fillPath of a
    2048^2-scaled heart with a linear gradient paint (the mask / gradient /
    MaskBlend / draw chain), GPU ms (CUDA events) beside the oracle."""
    import torch
    out = {}
    img = px.Image(2048, 2048)
    names = {3: "linear", 4: "radial", 5: "angular"}
    for kind, hs in PAINT_HANDLES.items():
        paint = px.Paint(kind=kind, handles=hs, stops=PAINT_STOPS)
        px.set_blocking(False)
        for _ in range(2):
            img.fill(paint)
        px.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            img.fill(paint)
        e1.record(stream)
        px.synchronize()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        row = {"gpu_ms": round(ms, 4), "gpix_per_s": round(2048 * 2048 / ms / 1e6, 2)}
        if cpu:  # the oracle, one thread, on a 512^2 image with the handles scaled by 1/4
            from oracle import pxo
            small = pxo.new_image(512, 512)
            t = time.perf_counter()
            pxo.fill_paint(small, dict(kind=kind, handles=[(x / 4, y / 4) for x, y in hs], stops=PAINT_STOPS))
            row["cpu_oracle_ms_scaled_to_2048"] = round((time.perf_counter() - t) * 1000 * 16, 1)
        out[f"fill_{names[kind]}_gradient"] = row
    heart = wl.heart_commands(20.48)
    paint = px.Paint(kind=3, handles=PAINT_HANDLES[3], stops=PAINT_STOPS, opacity=0.8)
    px.set_blocking(True)
    for _ in range(2):
        img.fill_path(heart, paint)
    t = time.perf_counter()
    for _ in range(reps):
        img.fill_path(heart, paint)
    dt = (time.perf_counter() - t) / reps * 1000
    out["fill_path_linear_gradient_heart"] = {"call_ms": round(dt, 3),
                                              "note": "one blocking call, 2048^2: mask fill + gradient + "
                                                      "MaskBlend + draw"}
    px.set_blocking(True)
    return out


def record_scene(px, items, threads=0):
    """Records the scene's paths in one batched call (geometry built on host
    threads, appended in order); returns the scene and the failed count."""
    sc = px.Scene()
    status = sc.record_batch(items, threads)
    return sc, int(status.sum())


def run_serving(px, wl, n_jobs, pool, rates=(5, 10, 100, 20000), seed=11):
    """Open-loop serving sweep: Poisson arrivals at each rate, n_jobs jobs per
    rate drawn from a pool of recorded jobs (canvas side log-U[256, 4096],
    10..5000 dense-scene paths, blur r in 2..32 on 20% of jobs), admitted
    against a 40 GB budget.  Latency = arrival -> canvas copied back to the
    host.  Every served canvas is compared with the same job rendered alone.
    Rates below the service capacity measure service latency; rates above it
    measure the drain of the queue.  Occupancy = device bytes the admitted
    jobs hold (sampled after every step) over the budget."""
    budget = 40 << 30
    t = time.perf_counter()
    seeds = [seed * 100 + k for k in range(pool)]
    jobs = [wl.serving_job(sd) for sd in seeds]
    scenes = [record_scene(px, j["items"])[0] for j in jobs]
    prep_s = time.perf_counter() - t
    alone = []
    alone_ms = []
    for j, sc in zip(jobs, scenes):
        img = px.Image(j["side"], j["side"])
        t = time.perf_counter()
        img.draw_scene(sc)
        if j["blur"]:
            img.blur(j["blur"])
        alone.append(img.to_numpy())
        alone_ms.append((time.perf_counter() - t) * 1e3)
    res = {"pool_jobs": pool, "jobs_per_rate": n_jobs, "budget_gb": 40, "pool_seeds": seeds,
           "pool_side_min_median_max": [min(j["side"] for j in jobs), int(np.median([j["side"] for j in jobs])),
                                        max(j["side"] for j in jobs)],
           "pool_paths_min_median_max": [min(len(s) for s in scenes), int(np.median([len(s) for s in scenes])),
                                         max(len(s) for s in scenes)],
           "pool_blurred": sum(1 for j in jobs if j["blur"]), "prep_s": round(prep_s, 1),
           "alone_ms_mean": round(float(np.mean(alone_ms)), 2),
           "service_capacity_jobs_per_s_est": round(1e3 / float(np.mean(alone_ms)), 2), "rates": []}
    all_exact = True
    for ri, rate in enumerate(rates):
        sv = px.Server(budget, 512, 16384)
        arr = wl.poisson_arrivals(seed + ri, float(rate), n_jobs)
        which = {}
        lat = []
        exact = True
        i = 0
        done = 0
        occ, adm = [], []
        step_host_s = 0.0
        t0 = time.perf_counter()
        while done < n_jobs:
            now = time.perf_counter() - t0
            while i < n_jobs and arr[i] <= now:
                k = i % pool
                jid = sv.submit(scenes[k], jobs[k]["side"], jobs[k]["side"], jobs[k]["blur"])
                which[jid] = (k, arr[i])
                i += 1
            if sv.pending() > 0:
                ts = time.perf_counter()
                sv.step()
                step_host_s += time.perf_counter() - ts
                st = sv.stats()
                occ.append(st["bytes_used"])
                adm.append(st["admitted"])
            elif i < n_jobs:
                time.sleep(max(0.0, min(arr[i] - (time.perf_counter() - t0), 0.002)))
            for jid in sv.poll():
                outimg, _ = sv.take(jid)
                k, a = which.pop(jid)
                lat.append(time.perf_counter() - t0 - a)
                exact = exact and outimg is not None and np.array_equal(outimg, alone[k])
                done += 1
        wall = time.perf_counter() - t0
        st = sv.stats()
        lat_ms = np.sort(np.asarray(lat)) * 1e3
        res["rates"].append({"rate_jobs_per_s": rate, "jobs": n_jobs,
                             "jobs_per_s": round(n_jobs / wall, 2),
                             "saturated": bool(n_jobs / wall < 0.9 * rate),
                             "p50_ms": round(float(np.percentile(lat_ms, 50)), 2),
                             "p99_ms": round(float(np.percentile(lat_ms, 99)), 2),
                             "steps": st["steps"], "peak_admitted": st["peak_admitted"],
                             "mean_admitted": round(float(np.mean(adm)), 2) if adm else 0.0,
                             "peak_gb": round(st["peak_bytes"] / 2**30, 3),
                             "budget_occupancy_mean": round(float(np.mean(occ)) / budget, 5) if occ else 0.0,
                             "budget_occupancy_peak": round(st["peak_bytes"] / budget, 5),
                             "step_call_share_of_wall": round(step_host_s / wall, 3),
                             "bitexact_vs_alone": bool(exact)})
        all_exact = all_exact and exact
        del sv
    res["all_bitexact_vs_alone"] = all_exact
    return res


def run_glyphs(px, wl, n, seed=7, page_side=4096, reps=5):
    """The glyph batch: n glyph outlines, each into its own 8-bit mask, then
    composited in order onto a page with NormalBlend.  Batched: one mask
    batch (recorded once; one graph launch renders it) + one ordered
    composite.  Plain: one blocking fillPath per glyph into its own image,
    then one draw per glyph."""
    glyphs, pos = wl.glyph_batch(seed, n=n, page=page_side)
    page = px.Image(page_side, page_side)
    t = time.perf_counter()  # one add_path call per glyph
    m1 = px.Masks()
    for cmds, w, h, wind in glyphs:
        m1.add_path(cmds, w, h, None, wind)
    rec1_s = time.perf_counter() - t
    del m1
    t = time.perf_counter()  # the same glyphs in one batched call (geometry on host threads)
    m = px.Masks()
    m.add_paths(glyphs)
    rec_s = time.perf_counter() - t
    m.render()  # first render of the class: the autotuner times its candidates
    page.draw_masks(m, pos)
    px.synchronize()
    render_ms, wall, comp_ms = [], [], []
    for _ in range(reps):
        page.fill([0, 0, 0, 0])
        px.synchronize()
        t = time.perf_counter()
        m.render()
        render_ms.append(px.last_gpu_ms())
        page.draw_masks(m, pos)
        px.synchronize()
        wall.append(time.perf_counter() - t)
    # composite alone, timed on the library's stream
    for _ in range(reps):
        t0 = time.perf_counter()
        page.draw_masks(m, pos)
        px.synchronize()
        comp_ms.append((time.perf_counter() - t0) * 1e3)
    imgs = [px.Image(w, h) for (_, w, h, _) in glyphs]
    for im, (c, _, _, wd) in zip(imgs[:64], glyphs[:64]):
        im.fill_path(c, [1, 1, 1, 1], None, wd)
    page.fill([0, 0, 0, 0])
    px.synchronize()
    t = time.perf_counter()
    for im, (c, _, _, wd), (x, y) in zip(imgs, glyphs, pos):
        im.fill_path(c, [1, 1, 1, 1], None, wd)
        page.draw(im, (int(x), int(y)))
    px.synchronize()
    dt_plain = time.perf_counter() - t
    b = sorted(wall)[len(wall) // 2]
    return {"glyphs": n, "page": f"{page_side}x{page_side}",
            "batched_paths_per_s": round(n / b, 1),
            "batched_incl_recording_paths_per_s": round(n / (b + rec_s), 1),
            "plain_paths_per_s": round(n / dt_plain, 1),
            "batched_over_plain": round(dt_plain / b, 2),
            "batched_incl_recording_over_plain": round(dt_plain / (b + rec_s), 2),
            "render_gpu_ms": round(sorted(render_ms)[len(render_ms) // 2], 3),
            "composite_call_ms": round(sorted(comp_ms)[len(comp_ms) // 2], 3),
            "record_ms_host": round(rec_s * 1e3, 1),
            "record_ms_host_one_call_per_glyph": round(rec1_s * 1e3, 1),
            "autotune": px.autotune_report().strip().splitlines(),
            "note": "batched = one graph launch rendering all masks + one ordered composite; "
                    "plain = blocking fillPath + draw per glyph"}


def run_svg_tiger(px, cpu=True, reps=5):
    """The Ghostscript tiger SVG (the reference's test document) through the SVG
    front-end: parse + record (host), then one scene draw of its 304 calls
    onto 900x900 (GPU), beside the oracle making the same calls one by one."""
    from pixie_gb300 import svg as S
    with np.load(os.path.join(ROOT, "tests", "golden", "inputs.npz")) as z:
        text = bytes(z["svg_Ghostscript_Tiger"]).decode("utf-8")
    t = time.perf_counter()
    d = S.parse_svg(text)
    parse_ms = (time.perf_counter() - t) * 1e3
    t = time.perf_counter()
    sc, status = S.svg_scene(d)
    record_ms = (time.perf_counter() - t) * 1e3
    img = px.Image(d.width, d.height)
    img.draw_scene(sc)  # first draw: upload and stroke outlines
    gpu, wall = [], []
    for _ in range(reps):
        img.fill([0, 0, 0, 0])
        t = time.perf_counter()
        img.draw_scene(sc)
        wall.append((time.perf_counter() - t) * 1e3)
        gpu.append(px.last_gpu_ms())
    out = {"calls": len(sc), "parse_ms_host": round(parse_ms, 1), "record_ms_host": round(record_ms, 1),
           "gpu_ms_per_draw": round(sorted(gpu)[reps // 2], 3), "draw_call_ms": round(sorted(wall)[reps // 2], 3)}
    if cpu:
        from oracle import pxo
        ref = pxo.new_image(d.width, d.height)
        t = time.perf_counter()
        for it in S.svg_items(d):
            if it["kind"] == "fill":
                pxo.fill_path(ref, it["cmds"], it["color"], it["opacity"], it["blend"], it["transform"],
                              it["winding"])
            else:
                pxo.stroke_path(ref, it["cmds"], it["color"], it["opacity"], it["blend"], it["transform"],
                                it["width"], it["cap"], it["join"], it["miter"], it["dashes"])
        out["cpu_oracle_ms_1core"] = round((time.perf_counter() - t) * 1e3, 1)
        out["bitexact_vs_oracle"] = bool(np.array_equal(img.to_numpy(), ref))
    return out


def run_scene(px, wl, seed=7, n_paths=2000, size=1024, reps=3):
    """The dense scene: 2000 mixed paths recorded (host geometry), then painted
    in order onto a 1024x1024 canvas by one draw_scene call."""
    items = wl.dense_scene(seed, n_paths=n_paths, size=float(size))
    t = time.perf_counter()  # one call per path, as a caller of the reference's API records
    sc1 = px.Scene()
    for it in items:
        paint = px.Paint(it["color"], 1.0, it["blend"])
        try:
            if it["kind"] == "fill":
                sc1.fill_path(it["cmds"], paint, None, it["winding"])
            else:
                sc1.stroke_path(it["cmds"], paint, None, it["width"], it["cap"], it["join"], it["miter"])
        except px.PixieError:
            pass  # arcs the reference's arc stepping cannot discretise
    rec1_s = time.perf_counter() - t
    del sc1
    t = time.perf_counter()  # the same paths in one batched call (geometry on host threads)
    sc, failed = record_scene(px, items)
    rec_s = time.perf_counter() - t
    canvas = px.Image(size, size)
    canvas.draw_scene(sc)
    stats = px.last_fill_stats()
    gpu_ms = []
    wall = []
    for _ in range(reps):
        canvas.fill([0, 0, 0, 0])
        t = time.perf_counter()
        canvas.draw_scene(sc)
        wall.append(time.perf_counter() - t)
        gpu_ms.append(px.last_gpu_ms())
    g = sorted(gpu_ms)[len(gpu_ms) // 2]
    w = sorted(wall)[len(wall) // 2]
    painted = len(sc)
    return {"paths_recorded": painted, "paths_raising_in_reference": failed,
            "segments": stats["segments"], "primitives": stats["primitives"],
            "covered_pixel_blends": stats["pixel_blends"], "wide_rows": stats["wide_rows"],
            "gpu_ms_per_scene": round(g, 3), "paths_per_s_gpu": round(painted / (g / 1e3), 1),
            "edges_per_s_gpu": round(stats["segments"] / (g / 1e3), 1),
            "covered_gpix_per_s_gpu": round(stats["pixel_blends"] / (g / 1e3) / 1e9, 3),
            "draw_call_ms": round(w * 1e3, 3), "record_ms_host": round(rec_s * 1e3, 1),
            "record_ms_host_one_call_per_path": round(rec1_s * 1e3, 1),
            "host_threads": os.cpu_count(),
            "note": "gpu_ms covers the primitive upload, setup and scene launches of draw_scene; "
                    "record_ms is the host command walk and stroke outlining of all paths "
                    "(one batched call, geometry on host threads)"}


# DRAM traffic per operation (dram__bytes_read.sum + dram__bytes_write.sum,
# summed over the operation's launches) from ncu captures of the same
# kernels: a blur of 4096x4096 at radius 16 or 64 = the two tensor-core ring
# passes (python bench.py --case blur16 / blur64, the first two launches).
TRAFFIC = {"blur:16": 67226368 + 13997312 + 67230464 + 12313856,
           "blur:64": 67218432 + 14129920 + 67217664 + 12249088}


# -- CPU baseline / reference arm ----------------------------------------------------------
def cpu_sample_rates(seed=1, simd=True):
    """Single-thread oracle throughput per operation on a bounded sample.
    simd: the Normal/Mask/Overwrite lines run the oracle's restatement of the
    reference's NEON kernels (what a pixie build on this host runs: the
    reference's blur and other blend modes are scalar on every ISA).
    Returns (estimated seconds for one full step, description)."""
    from oracle import pxo
    from pixie_gb300 import workloads as wl
    pxo.set_simd_variant(simd)
    try:
        return _cpu_sample(seed, simd, pxo, wl)
    finally:
        pxo.set_simd_variant(False)


def _cpu_sample(seed, simd, pxo, wl):
    S = 1024
    a = wl.premultiplied_image(seed * 10, S, S)
    b = wl.premultiplied_image(seed * 10 + 5, S, S)
    est = 0.0
    for mode in range(N_MODES):
        x = a.copy()
        t = time.perf_counter()
        pxo.draw(x, b, 0, 0, mode)
        dt = time.perf_counter() - t
        est += dt * (DRAW_W * DRAW_W) / (S * S)
    bl = wl.premultiplied_image(seed * 10 + 9, 1024, 384)
    for r in RADII:
        x = bl.copy()
        t = time.perf_counter()
        pxo.blur(x, r)
        dt = time.perf_counter() - t
        est += dt * (BLUR_W * BLUR_W) / x[..., 0].size
    mask = pxo.new_image(SHADOW_W, SHADOW_W)
    pxo.fill_path(mask, wl.disc_mask_path(seed), [1, 1, 1, 1])
    t = time.perf_counter()
    pxo.shadow(mask, 8, 8, 4, 12, [0, 0, 0, 1])
    est += time.perf_counter() - t
    what = ("C++ restatement of pixie's SIMD build (its NEON line kernels for Normal/Mask lines, "
            "scalar elsewhere as in pixie)" if simd else "C++ restatement of pixie's scalar path")
    return est, (what + ", 1 thread: draw 20 modes on 1024^2, blur r in {1,4,16,64} on 1024x384, "
                 "shadow on 1024^2; scaled per pixel to the full step")


def _ref_worker(args):
    seed, simd = args
    sys.path.insert(0, ROOT)
    est, _ = cpu_sample_rates(seed, simd)
    return est


def host_info():
    import platform
    return {"uname_m": platform.machine(), "nproc": os.cpu_count()}


def run_reference(args, ws, rank):
    if rank != 0:
        return None
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        for _ in range(args.warmup):
            pool.map(_ref_worker, [(k, True) for k in range(1, cores + 1)])
        t = time.perf_counter()
        est_total = 0.0
        for _ in range(args.steps):
            ests = pool.map(_ref_worker, [(k, True) for k in range(1, cores + 1)])
            est_total += statistics.mean(ests)
        wall = time.perf_counter() - t
        scalar = statistics.mean(pool.map(_ref_worker, [(k, False) for k in range(1, cores + 1)]))
    per_step_single = est_total / args.steps
    value = STEP_PIXELS * cores / per_step_single / 1e9  # cores run independent steps
    return {"value": value, "cores": cores, "wall_s": wall,
            "ms_per_step": per_step_single * 1e3 / cores,
            "scalar_value": STEP_PIXELS * cores / scalar / 1e9}


def run_case(case: str, slice_w: int = 0):
    """One small, self-contained invocation of a single operation (used for
    ncu captures of one kernel on a small case)."""
    import pixie_gb300 as px
    from pixie_gb300 import workloads as wl
    px.lib().pxg_init(0)
    if case == "fill512":  # the plain fill: 512x512, 64 random cubics
        img = px.Image(512, 512)
        for s in (1, 2, 3):
            img.fill_path(wl.plain_path(s), wl.PLAIN_COLOR)
    elif case.startswith("blur"):  # blur<r>: two blurs of radius r (default 64) of a 4096x4096 image
        r = int(case[4:] or 64)
        img = px.Image.from_numpy(wl.premultiplied_image(9, 4096, 4096))
        for _ in range(2):
            img.blur(r)
    elif case.startswith("draw"):  # draw<mode>: a 4096x4096 draw onto 4096x4096 (inputs > L2), default Normal
        mode = int(case[4:] or 0)
        a = px.Image.from_numpy(wl.premultiplied_image(1, 4096, 4096))
        b = px.Image.from_numpy(wl.premultiplied_image(2, 4096, 4096))
        for _ in range(2):
            a.draw(b, (0, 0), mode)
    elif case == "paint":  # 2048^2: a fill with each gradient kind, then fillPath of a heart with a linear gradient
        img = px.Image(2048, 2048)
        for kind, hs in PAINT_HANDLES.items():
            img.fill(px.Paint(kind=kind, handles=hs, stops=PAINT_STOPS))
        img.fill_path(wl.heart_commands(20.48), px.Paint(kind=3, handles=PAINT_HANDLES[3], stops=PAINT_STOPS,
                                                         opacity=0.8))
    elif case == "smooth":  # draw of a 2048^2 source rotated 30 degrees, scaled 1.1, onto 2048^2
        a = px.Image.from_numpy(wl.premultiplied_image(1, 2048, 2048))
        b = px.Image.from_numpy(wl.premultiplied_image(2, 2048, 2048))
        for _ in range(2):
            a.draw_transform(b, smooth_mat(*SMOOTH_CASES["rotate30_scale1.1"][0]), 0)
    elif case == "glyphs":  # batched fill of 512 glyph masks
        glyphs, _ = wl.glyph_batch(7, n=512)
        imgs = [px.Image(w, h) for (_, w, h, _) in glyphs]
        for _ in range(2):
            px.fill_paths_batch(imgs, [g[0] for g in glyphs], [[1, 1, 1, 1]] * len(glyphs),
                                winding_rules=[g[3] for g in glyphs])
    elif case in ("scene", "scene_small", "scene_normal"):
        # dense scene: 2000 paths on 1024^2 (small: 400 on 512^2; normal: every path NormalBlend)
        n, side = (400, 512) if case == "scene_small" else (2000, 1024)
        if slice_w:
            px.scene_config(slice_w)
        items = wl.dense_scene(7, n_paths=n, size=float(side))
        if case == "scene_normal":
            for it in items:
                it["blend"] = 0
        sc, _ = record_scene(px, items)
        img = px.Image(side, side)
        for _ in range(2):
            img.draw_scene(sc)
        print(json.dumps(px.last_fill_stats()))
    elif case == "masks":  # 4096 glyph masks rendered, then composited onto a 4096^2 page
        glyphs, pos = wl.glyph_batch(7, n=4096)
        m = px.Masks()
        for cmds, w, h, wind in glyphs:
            m.add_path(cmds, w, h, None, wind)
        px.autotune(False)
        page = px.Image(4096, 4096)
        for _ in range(2):
            m.render()
            page.draw_masks(m, pos)
    else:
        raise SystemExit(f"unknown case {case}")
    px.synchronize()
    print(json.dumps({"case": case, "launches": px.launch_count()}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="pxg", choices=["pxg", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--glyphs", type=int, default=4096)
    ap.add_argument("--serve-jobs", type=int, default=200, help="jobs per arrival rate (0: skip serving)")
    ap.add_argument("--serve-pool", type=int, default=100, help="distinct recorded jobs the arrivals draw from")
    ap.add_argument("--no-fill", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the oracle comparison of the step's outputs")
    ap.add_argument("--serve-rates", default="5,10,100,20000",
                    help="comma-separated Poisson arrival rates (jobs/s) of the serving sweep")
    ap.add_argument("--slice", type=int, default=0, help="scene row slice width for --case scene*")
    ap.add_argument("--case", default=None,
                    help="run one small operation for profiling: fill512 | blur<r> (blur64) | draw<mode> (draw13) | smooth | paint | glyphs | scene | scene_small | masks")
    args = ap.parse_args()
    if args.case:
        run_case(args.case, args.slice)
        return
    ws, rank, local = dist_setup()

    if args.impl == "reference":
        r = run_reference(args, ws, rank)
        if rank == 0:
            line = {"metric": METRIC, "value": round(r["value"], 4), "unit": "Gpix/s",
                    "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
                    "ms_per_step": round(r["ms_per_step"], 3), "higher_is_better": True,
                    "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
                    "config": WORKLOAD, "impl": "reference",
                    "cpu_baseline": {"value": round(r["value"], 4), "unit": "Gpix/s",
                                     "cores": r["cores"], "kind": "port",
                                     "scalar_value": round(r["scalar_value"], 4),
                                     "sample": "per core: draw 20 modes on 1024^2, blur r in "
                                               "{1,4,16,64} on 1024x384, shadow 1024^2, scaled "
                                               "per pixel; pixie (Nim) cannot be built here, so "
                                               "this is the oracle's C++ restatement of pixie's SIMD "
                                               "build (NEON line kernels on aarch64; scalar_value: "
                                               "the scalar build)", **host_info()},
                    "e2e": {"value": round(r["value"], 4), "unit": "Gpix/s",
                            "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
            print(json.dumps(line), flush=True)
        return

    ms_step, launches, roof, e2e, extra, clocks, parity = run_gpu(args, ws, rank, local)
    if rank != 0:
        return
    value = STEP_PIXELS * ws / (ms_step * 1e-3) / 1e9
    cpu = None
    if not args.no_cpu_baseline:
        est, sample = cpu_sample_rates(1)
        est_scalar, _ = cpu_sample_rates(1, simd=False)
        cpu = {"value": round(STEP_PIXELS / est / 1e9, 5), "unit": "Gpix/s", "cores": 1,
               "kind": "port", "sample": sample, "scalar_value": round(STEP_PIXELS / est_scalar / 1e9, 5),
               **host_info()}
    line = {"metric": METRIC, "value": round(value, 3), "unit": "Gpix/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u8",
            "data": "synthetic (seeded splitmix64; shapes/distributions of the configuration)",
            "config": WORKLOAD, "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(launches), "clocks": clocks, "parity": parity, "extra": extra}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
