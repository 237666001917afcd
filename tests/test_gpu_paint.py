"""Non-solid paints on the CUDA library against the oracle, bit for bit:
gradients (linear, radial, angular), image and tiled image paints, fillPath /
strokePath with them, fill with a paint, drawTiled, and the reference's errors.
The reference's own paint scenes run in test_gpu_parity's golden-scene test.
"""
import math

import numpy as np
import pytest

import pixie_gb300 as px
from cases import HEART
from oracle import pxo
from pixie_gb300 import workloads as wl
from pixie_gb300.paths import parse_path

pytestmark = pytest.mark.gpu

LINEAR, RADIAL, ANGULAR = 3, 4, 5


@pytest.fixture(scope="module", autouse=True)
def _init():
    px.lib().pxg_init(0)
    pxo.set_golden_mode(False)


def assert_same(gpu, cpu, what=""):
    gpu = np.asarray(gpu).astype(np.int32)
    cpu = np.asarray(cpu).astype(np.int32)
    assert gpu.shape == cpu.shape, what
    d = np.abs(gpu - cpu)
    n = int((d.reshape(-1, 4).max(axis=1) > 0).sum())
    assert n == 0, f"{what}: max|delta|={int(d.max())} differing px={n}"


def f32(v):
    return float(np.float32(v))


def rand_stops(rng, n):
    pos = sorted(f32(v) for v in rng.uniform(-0.2, 1.2, n))
    return [(tuple(f32(v) for v in rng.uniform(0, 1, 4)), p) for p in pos]


def rand_gradient(rng, kind, w, h):
    nh = 2 if kind == LINEAR else 3
    handles = [(f32(rng.uniform(-20, w + 20)), f32(rng.uniform(-20, h + 20))) for _ in range(nh)]
    return dict(kind=kind, handles=handles, stops=rand_stops(rng, int(rng.integers(1, 6))),
                opacity=f32(rng.choice([1.0, 0.5, 0.3, 0.99])), blend=int(rng.integers(0, 20)))


def gpu_paint(d, image=None):
    return px.Paint(d.get("color", (0, 0, 0, 0)), d.get("opacity", 1.0), d.get("blend", 0), kind=d["kind"],
                    image=image, image_mat=d.get("image_mat"), handles=d.get("handles", ()),
                    stops=d.get("stops", ()))


def heart():
    return parse_path(HEART).array()


def both_fill_path(dst, cmds, paint, src=None, mat=None, winding=0):
    ref = dst.copy()
    d = dict(paint)
    if src is not None:
        d["image"] = src
    pxo.fill_path_paint(ref, cmds, d, mat, winding)
    img = px.Image.from_numpy(dst)
    img.fill_path(cmds, gpu_paint(paint, px.Image.from_numpy(src) if src is not None else None), mat, winding)
    return img.to_numpy(), ref


@pytest.mark.parametrize("kind", [LINEAR, RADIAL, ANGULAR])
@pytest.mark.parametrize("seed", range(8))
def test_gradient_fill_path(kind, seed):
    rng = np.random.default_rng(1000 * kind + seed)
    dst = wl.premultiplied_image(seed + 3, 120, 100)
    paint = rand_gradient(rng, kind, 120, 100)
    mat = [f32(v) for v in (1.1, 0.1, 0, -0.1, 0.9, 0, rng.uniform(0, 20), rng.uniform(0, 10), 1)]
    gpu, ref = both_fill_path(dst, heart(), paint, mat=mat, winding=seed % 2)
    assert_same(gpu, ref, f"kind {kind} seed {seed}")


@pytest.mark.parametrize("kind", [LINEAR, RADIAL, ANGULAR])
def test_gradient_fill_paint_large(kind):
    """fill(image, gradient) writes the gradient itself; 1024x1024"""
    rng = np.random.default_rng(77 + kind)
    paint = rand_gradient(rng, kind, 1024, 1024)
    paint["stops"] = rand_stops(rng, 5)
    ref = pxo.new_image(1024, 1024)
    pxo.fill_paint(ref, paint)
    img = px.Image(1024, 1024)
    img.fill(gpu_paint(paint))
    assert_same(img.to_numpy(), ref, f"kind {kind}")


def test_angular_gradient_atan2_matches():
    """the shared float-float arctangent: every pixel of a 1500x1500 angular
    gradient whose stops turn each ulp of t into a colour step"""
    stops = [((0.0, 0.0, 0.0, 1.0), 0.0), ((1.0, 1.0, 1.0, 1.0), 1.0)]
    paint = dict(kind=ANGULAR, handles=[(f32(749.5), f32(750.25)), (f32(1400.0), f32(700.0)), (0.0, 0.0)],
                 stops=stops)
    ref = pxo.new_image(1500, 1500)
    pxo.fill_paint(ref, paint)
    img = px.Image(1500, 1500)
    img.fill(gpu_paint(paint))
    assert_same(img.to_numpy(), ref, "angular 1500^2")


@pytest.mark.parametrize("kind", [LINEAR, RADIAL, ANGULAR])
@pytest.mark.parametrize("nstops", [2457, 2458, 3000])
def test_gradient_many_stops(kind, nstops):
    """gradientColor takes any number of stops: up to 2457 (48 KB) the kernel
    stages them in shared memory, beyond that it reads them from global memory"""
    rng = np.random.default_rng(nstops + kind)
    paint = rand_gradient(rng, kind, 300, 200)
    paint["stops"] = rand_stops(rng, nstops)
    ref = pxo.new_image(300, 200)
    pxo.fill_paint(ref, paint)
    img = px.Image(300, 200)
    img.fill(gpu_paint(paint))
    assert_same(img.to_numpy(), ref, f"kind {kind}, {nstops} stops")


@pytest.mark.parametrize("tiled", [False, True])
@pytest.mark.parametrize("seed", range(6))
def test_image_paint(tiled, seed):
    rng = np.random.default_rng(50 + seed + 10 * tiled)
    src = wl.premultiplied_image(seed + 40, int(rng.integers(16, 90)), int(rng.integers(16, 90)))
    a = math.radians(rng.uniform(-180, 180))
    s = rng.choice([0.05, 0.3, 0.7, 1.0, 1.6, 3.0])
    tx, ty = rng.uniform(-60, 60, 2)
    mat = [f32(v) for v in (math.cos(a) * s, math.sin(a) * s, 0, -math.sin(a) * s, math.cos(a) * s, 0, tx, ty, 1)]
    paint = dict(kind=2 if tiled else 1, image_mat=mat, opacity=f32(rng.choice([1.0, 0.5, 0.8])),
                 blend=int(rng.integers(0, 20)))
    dst = wl.premultiplied_image(seed + 90, 110, 90)
    gpu, ref = both_fill_path(dst, heart(), paint, src=src)
    assert_same(gpu, ref, f"tiled={tiled} seed {seed}")


@pytest.mark.parametrize("kind", [1, 2])
def test_fill_with_image_paint(kind):
    src = wl.premultiplied_image(5, 64, 48)
    paint = dict(kind=kind, image_mat=[f32(v) for v in (0.37, 0, 0, 0, 0.41, 0, -3.5, 7.25, 1)], opacity=f32(0.5))
    dst = wl.premultiplied_image(6, 128, 96)
    ref = dst.copy()
    d = dict(paint)
    d["image"] = src
    pxo.fill_paint(ref, d)
    img = px.Image.from_numpy(dst)
    img.fill(gpu_paint(paint, px.Image.from_numpy(src)))
    assert_same(img.to_numpy(), ref, f"kind {kind}")


@pytest.mark.parametrize("kind", [1, 2, LINEAR, RADIAL, ANGULAR])
def test_stroke_path_paint(kind):
    rng = np.random.default_rng(kind)
    src = wl.premultiplied_image(8, 50, 50)
    paint = rand_gradient(rng, kind, 100, 100) if kind >= 3 else dict(
        kind=kind, image_mat=[f32(v) for v in (0.5, 0.2, 0, -0.2, 0.5, 0, 10, 5, 1)], opacity=f32(0.7), blend=2)
    dst = wl.premultiplied_image(9, 100, 100)
    cmds = parse_path("M 10 10 L 90 30 L 40 90 Z M 60 60 L 95 95").array()
    ref = dst.copy()
    d = dict(paint)
    if kind < 3:
        d["image"] = src
    pxo.stroke_path_paint(ref, cmds, d, width=f32(6.5), cap=1, join=2)
    img = px.Image.from_numpy(dst)
    img.stroke_path(cmds, gpu_paint(paint, px.Image.from_numpy(src) if kind < 3 else None),
                    stroke_width=6.5, line_cap=1, line_join=2)
    assert_same(img.to_numpy(), ref, f"kind {kind}")


@pytest.mark.parametrize("mode", [0, 3, 8, 16, 17, 19])
@pytest.mark.parametrize("mat", [(0.25, 0, 0, 0, 0.25, 0, 0, 0, 1), (0.6, 0.3, 0, -0.3, 0.6, 0, -40.5, 17.25, 1),
                                 (3.0, 0, 0, 0, 2.0, 0, 5, 5, 1), (1, 0, 0, 0, 1, 0, -7, -9, 1)])
def test_draw_tiled(mode, mat):
    src = wl.premultiplied_image(11, 37, 23)
    dst = wl.premultiplied_image(12, 90, 70)
    m = [f32(v) for v in mat]
    ref = dst.copy()
    pxo.draw_tiled(ref, src, m, mode)
    img = px.Image.from_numpy(dst)
    img.draw_tiled(px.Image.from_numpy(src), m, mode)
    assert_same(img.to_numpy(), ref, f"mode {mode} mat {mat}")


@pytest.mark.parametrize("paint,msg", [
    (dict(kind=LINEAR, handles=[(0.0, 0.0)], stops=[((1.0, 0.0, 0.0, 1.0), 0.0)]), "Linear gradient requires 2 handles"),
    (dict(kind=RADIAL, handles=[(0.0, 0.0), (1.0, 1.0)], stops=[((1.0, 0.0, 0.0, 1.0), 0.0)]),
     "Radial gradient requires 3 handles"),
    (dict(kind=ANGULAR, handles=[(0.0, 0.0), (1.0, 1.0)], stops=[((1.0, 0.0, 0.0, 1.0), 0.0)]),
     "Angular gradient requires 2 handles"),
    (dict(kind=LINEAR, handles=[(0.0, 0.0), (1.0, 1.0)], stops=[]), "Gradient must have at least 1 color stop"),
])
def test_gradient_errors(paint, msg):
    with pytest.raises(pxo.OracleError, match=msg):
        pxo.fill_paint(pxo.new_image(8, 8), paint)
    with pytest.raises(px.PixieError, match=msg):
        px.Image(8, 8).fill(gpu_paint(paint))


@pytest.mark.parametrize("kind", [LINEAR, RADIAL, ANGULAR])
@pytest.mark.parametrize("stops,handles,opacity", [
    # two stops at the same position, a t that lands exactly on a stop (x = 50 of a 0..100 gradient)
    ([((1.0, 0.0, 0.0, 1.0), 0.0), ((0.0, 1.0, 0.0, 1.0), 0.5), ((0.0, 0.0, 1.0, 1.0), 0.5),
      ((1.0, 1.0, 0.0, 0.5), 1.0)], [(0.0, 50.0), (100.0, 50.0), (0.0, 100.0)], 1.0),
    # stops outside 0..1 and out of order
    ([((0.2, 0.4, 0.6, 0.8), -0.5), ((0.9, 0.1, 0.3, 0.7), 1.5), ((0.5, 0.5, 0.5, 1.0), 0.25)],
     [(10.0, 10.0), (90.0, 70.0), (10.0, 90.0)], 0.75),
    # coincident handles: t is NaN (linear) or the matrix is singular (radial)
    ([((1.0, 0.0, 0.0, 1.0), 0.0), ((0.0, 0.0, 1.0, 1.0), 1.0)], [(50.0, 50.0), (50.0, 50.0), (50.0, 50.0)], 1.0),
    # a single stop, opacity above 1 (clamped)
    ([((0.3, 0.6, 0.9, 0.4), 0.7)], [(0.0, 0.0), (100.0, 100.0), (0.0, 100.0)], 1.7),
    # opacity 0 draws nothing
    ([((0.3, 0.6, 0.9, 0.4), 0.0), ((0.1, 0.2, 0.3, 1.0), 1.0)], [(0.0, 0.0), (100.0, 0.0), (0.0, 100.0)], 0.0),
])
def test_gradient_edges(kind, stops, handles, opacity):
    st = [(tuple(f32(c) for c in col), f32(p)) for col, p in stops]
    hs = [(f32(x), f32(y)) for x, y in handles[:2 if kind == LINEAR else 3]]
    paint = dict(kind=kind, handles=hs, stops=st, opacity=f32(opacity))
    dst = wl.premultiplied_image(5, 100, 100)
    ref = dst.copy()
    try:
        pxo.fill_paint(ref, paint)
    except pxo.OracleError as e:
        with pytest.raises(px.PixieError, match=str(e)):
            px.Image.from_numpy(dst).fill(gpu_paint(paint))
        return
    img = px.Image.from_numpy(dst)
    img.fill(gpu_paint(paint))
    assert_same(img.to_numpy(), ref, f"kind {kind}")
    # and through fillPath's paint chain
    gpu, ref2 = both_fill_path(dst, heart(), paint)
    assert_same(gpu, ref2, f"fillPath kind {kind}")
