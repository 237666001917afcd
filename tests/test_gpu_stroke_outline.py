"""Stroke outlines built on the GPU (strokeShapes, src/pixie/paths.nim:1922-2082)
against the oracle and against the host outline, byte for byte: every cap and
join, open and closed polylines with curves and arcs, transforms, scenes, and
joins built on purpose with turning angles at the decision thresholds (a
straight join's epsilon, the miter limit, the side of the turn), where the
library rebuilds the join on the host with the C library's atan2f."""
import math

import numpy as np
import pytest

import pixie_gb300 as px
from oracle import pxo
from pixie_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
PI = 3.141592653589793
EPS = float(np.float32(0.0001 * PI))


@pytest.fixture(scope="module", autouse=True)
def _init():
    px.lib().pxg_init(0)
    pxo.set_golden_mode(False)
    px.stroke_config(True)
    yield
    px.stroke_config(True)


def assert_same(gpu, cpu, what=""):
    d = np.abs(np.asarray(gpu).astype(np.int32) - np.asarray(cpu).astype(np.int32))
    n = int((d.reshape(-1, 4).max(axis=1) > 0).sum())
    assert n == 0, f"{what}: max|delta|={int(d.max())} differing px={n}"


def stroke_both(cmds, w, h, color, width, cap, join, miter=4.0, mat=None, blend=0, bg=None):
    """(GPU outline, host outline, oracle) of one strokePath call"""
    base = pxo.new_image(w, h) if bg is None else bg
    ref = base.copy()
    pxo.stroke_path(ref, cmds, color, 1.0, blend, mat, width, cap, join, miter)
    out = {}
    for gpu in (True, False):
        px.stroke_config(gpu)
        try:
            img = px.Image.from_numpy(base)
            img.stroke_path(cmds, px.Paint(color, 1.0, blend), mat, width, cap, join, miter)
            out[gpu] = img.to_numpy()
        finally:
            px.stroke_config(True)
    return out[True], out[False], ref


@pytest.mark.parametrize("cap", [0, 1, 2])
@pytest.mark.parametrize("join", [0, 1, 2])
@pytest.mark.parametrize("seed", range(3))
def test_random_strokes_every_cap_and_join(cap, join, seed):
    items = wl.dense_scene(900 + seed, n_paths=6, size=300.0)
    rng = np.random.default_rng(seed * 9 + cap * 3 + join)
    bg = wl.premultiplied_image(seed + 40, 300, 260)
    for k, it in enumerate(items):
        cmds = it["cmds"] if k % 2 == 0 else np.append(it["cmds"], np.float32(0.0))  # open and closed
        width = float(np.float32(rng.uniform(0.3, 12.0)))
        mat = None if k % 3 else [float(np.float32(v)) for v in (0.9, 0.2, 0, -0.1, 1.1, 0, 7.5, -3.25, 1)]
        try:
            gpu, host, ref = stroke_both(cmds, 300, 260, it["color"], width, cap, join, 4.0, mat,
                                         blend=it["blend"], bg=bg)
        except (px.PixieError, pxo.OracleError):
            continue  # the reference's arc stepping raises for this path
        assert_same(host, ref, f"host outline seed {seed} path {k}")
        assert_same(gpu, ref, f"GPU outline seed {seed} path {k}")


def polyline(points, closed=False):
    c = [1.0, float(points[0][0]), float(points[0][1])]
    for x, y in points[1:]:
        c += [2.0, float(x), float(y)]
    if closed:
        c.append(0.0)
    return np.asarray(c, np.float32)


def turn_subpaths(turns, side=700, arm=12.0):
    """one open three-point subpath per turn, on a grid: the segments meet at
    the grid point and the second turns by the given angle"""
    cols = int(math.ceil(math.sqrt(len(turns))))
    step = (side - 4 * arm) / cols
    c = []
    for k, t in enumerate(turns):
        cx, cy = 2 * arm + step * (k % cols), 2 * arm + step * (k // cols)
        pts = [(cx - arm, cy), (cx, cy), (cx + arm * math.cos(t), cy + arm * math.sin(t))]
        pts = [(float(np.float32(x)), float(np.float32(y))) for x, y in pts]
        c += [1.0, pts[0][0], pts[0][1], 2.0, pts[1][0], pts[1][1], 2.0, pts[2][0], pts[2][1]]
    return np.asarray(c, np.float32)


@pytest.mark.parametrize("join", [0, 2])
def test_joins_at_the_decision_thresholds(join):
    """Turning angles at the straight-join epsilon (|angle| = pi - eps), the
    miter limit (|angle| = 2 asin(1/4)) and a reversal (angle = 0), each within
    a few ulps: the GPU's decisions there are rebuilt with the C library."""
    miter_angle = float(np.float32(np.arcsin(np.float32(0.25)) * 2))
    turns = []
    for k in range(-40, 41):
        d = k * 2.5e-7
        turns += [EPS + d, -(EPS + d), PI - miter_angle + d, -(PI - miter_angle + d), PI - 1e-6 + d]
    cmds = turn_subpaths(turns)
    before = px.stroke_fixups()
    gpu, host, ref = stroke_both(cmds, 700, 700, [0.2, 0.6, 0.9, 0.8], 2.5, 0, join)
    assert px.stroke_fixups() > before  # the ambiguous joins went through the host
    assert_same(host, ref, "host outline")
    assert_same(gpu, ref, "GPU outline at the thresholds")


def test_scene_strokes_gpu_equals_host_and_oracle():
    items = wl.dense_scene(77, n_paths=120, size=400.0)
    ref = pxo.new_image(400, 400)
    pxo.draw_items(ref, items, 4)
    out = {}
    for gpu in (True, False):
        px.stroke_config(gpu)
        try:
            sc = px.Scene()
            sc.record_batch(items, 0)
            img = px.Image(400, 400)
            img.draw_scene(sc)
            out[gpu] = img.to_numpy()
        finally:
            px.stroke_config(True)
    assert_same(out[False], ref, "scene, host outlines")
    assert_same(out[True], ref, "scene, GPU outlines")


def test_single_stroke_recordings_and_mask_blend_strokes():
    """pxg_scene_stroke_path one call at a time, with MaskBlend strokes (which
    keep the host outline) between GPU-outlined ones"""
    items = wl.dense_scene(78, n_paths=40, size=256.0)
    for k, it in enumerate(items):
        if it["kind"] == "stroke" and k % 5 == 0:
            it["blend"] = 16
    bg = wl.premultiplied_image(3, 256, 256)
    ref = bg.copy()
    pxo.draw_items(ref, items, 1)
    sc = px.Scene()
    for it in items:
        paint = px.Paint(it["color"], 1.0, it["blend"])
        try:
            if it["kind"] == "fill":
                sc.fill_path(it["cmds"], paint, None, it["winding"])
            else:
                sc.stroke_path(it["cmds"], paint, None, it["width"], it["cap"], it["join"], it["miter"])
        except px.PixieError:
            pass
    img = px.Image.from_numpy(bg)
    img.draw_scene(sc)
    assert_same(img.to_numpy(), ref, "scene of single recordings")


def test_dashes_and_zero_width_keep_their_behaviour():
    cmds = polyline([(10, 10), (180, 40), (60, 170), (20, 90)])
    ref = pxo.new_image(200, 200)
    pxo.stroke_path(ref, cmds, [1, 0, 0, 1], 1.0, 0, None, 5.0, 1, 0, 4.0, (6.0, 3.0))
    img = px.Image(200, 200)
    img.stroke_path(cmds, px.Paint([1, 0, 0, 1], 1.0, 0), None, 5.0, 1, 0, 4.0, (6.0, 3.0))
    assert_same(img.to_numpy(), ref, "dashed stroke (host outline)")
    # a zero-width stroke has no outline: the reference's fillShapes then
    # raises on the empty bounds, and so does the library
    with pytest.raises(pxo.OracleError, match="Path int overflow detected"):
        pxo.stroke_path(pxo.new_image(200, 200), cmds, [1, 0, 0, 1], 1.0, 0, None, 0.0, 1, 0)
    with pytest.raises(px.PixieError, match="Path int overflow detected"):
        px.Image(200, 200).stroke_path(cmds, px.Paint([1, 0, 0, 1], 1.0, 0), None, 0.0, 1, 0)
