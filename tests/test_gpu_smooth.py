"""draw with a Mat3 transform (drawSmooth, minifyBy2, magnifyBy2) on the CUDA
library against the oracle, bit for bit.

The reference's own scenes (rotate*, scaleHalf, smooth*, minify_odd,
rock_minified*) run in test_gpu_parity's golden-scene test; here: random
affine transforms over every blend mode, transforms that take the minify and
magnify pre-passes, whole-pixel translations (blendRect), MaskBlend's
clearing, degenerate transforms and the resampling entry points.
"""
import math

import numpy as np
import pytest

import pixie_gb300 as px
from oracle import pxo
from pixie_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

MODES = list(range(20))


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


def affine(angle_deg, sx, sy, tx, ty):
    """translate(tx, ty) * rotate(angle) * scale(sx, sy) as a column-major Mat3,
    built in float64 and rounded to float32 (the product's rounding does not
    matter here: both sides receive the same nine floats)."""
    a = math.radians(angle_deg)
    c, s = math.cos(a), math.sin(a)
    return [f32(c * sx), f32(s * sx), 0.0, f32(-s * sy), f32(c * sy), 0.0, f32(tx), f32(ty), 1.0]


def run_both(dst, src, mat, mode):
    ref = dst.copy()
    pxo.draw_transform(ref, src, mat, mode)
    a = px.Image.from_numpy(dst)
    b = px.Image.from_numpy(src)
    a.draw_transform(b, mat, mode)
    return a.to_numpy(), ref


def rand_case(seed, w, h, bw, bh):
    return (wl.premultiplied_image(seed, w, h), wl.premultiplied_image(seed + 1000, bw, bh))


# random rotations, scales between 0.6 and 1.8 (no pre-pass), fractional offsets
@pytest.mark.parametrize("mode", MODES)
def test_random_affine_every_mode(mode):
    rng = np.random.default_rng(100 + mode)
    for k in range(3):
        dst, src = rand_case(7 * mode + k, 160, 120, int(rng.integers(20, 90)), int(rng.integers(20, 90)))
        mat = affine(rng.uniform(-180, 180), rng.uniform(0.6, 1.8), rng.uniform(0.6, 1.8),
                     rng.uniform(-30, 150), rng.uniform(-30, 110))
        gpu, ref = run_both(dst, src, mat, mode)
        assert_same(gpu, ref, f"mode {mode} case {k}")


@pytest.mark.parametrize("scale", [0.03, 0.1, 0.24, 0.26, 0.49, 0.5, 0.51, 1.99, 2.0, 2.01, 3.7, 9.0])
@pytest.mark.parametrize("mode", [0, 16, 17])
def test_minify_and_magnify_prepasses(scale, mode):
    dst, src = rand_case(int(scale * 100) + mode, 200, 150, 123, 77)
    mat = affine(17.0, scale, scale, 11.5, 7.25)
    gpu, ref = run_both(dst, src, mat, mode)
    assert_same(gpu, ref, f"scale {scale} mode {mode}")


@pytest.mark.parametrize("t", [(0, 0), (5, 9), (-7, 3), (0.5, 0.5), (25.2, 25.6), (-3.75, 11.0), (1e-3, 0)])
@pytest.mark.parametrize("mode", [0, 3, 12, 16, 17, 19])
def test_translations(t, mode):
    dst, src = rand_case(31, 90, 70, 40, 30)
    mat = [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, f32(t[0]), f32(t[1]), 1.0]
    gpu, ref = run_both(dst, src, mat, mode)
    assert_same(gpu, ref, f"translate {t} mode {mode}")


def test_fractional_translate_through_draw():
    """draw(b, (x, y)) with a fractional offset takes drawSmooth"""
    dst, src = rand_case(5, 64, 64, 20, 20)
    ref = dst.copy()
    pxo.draw_transform(ref, src, [1, 0, 0, 0, 1, 0, 10.5, 3.25, 1], 0)
    a = px.Image.from_numpy(dst)
    a.draw(px.Image.from_numpy(src), (10.5, 3.25), 0)
    assert_same(a.to_numpy(), ref)


@pytest.mark.parametrize("mat", [
    [1, 0, 0, 0, 1, 0, 5000, 5000, 1],       # far outside
    [1, 0, 0, 0, 1, 0, -5000, 20, 1],
    [0.0, 0, 0, 0, 1, 0, 10, 10, 1],          # singular: zero x scale
    [0.0, 0, 0, 0, 0, 0, 10, 10, 1],          # singular: zero
    [1, 0, 0, 0, 1e-30, 0, 10, 10, 1],        # nearly singular
    [-1, 0, 0, 0, -1, 0, 80, 60, 1],          # flips
    [1, 0, 0, 0, -1, 0, 0, 60, 1],
    [0.7, 0.7, 0, -0.7, 0.7, 0, 40, -10, 1],
])
@pytest.mark.parametrize("mode", [0, 16, 17])
def test_edge_transforms(mat, mode):
    dst, src = rand_case(77, 96, 64, 50, 40)
    m = [f32(v) for v in mat]
    try:
        ref = dst.copy()
        pxo.draw_transform(ref, src, m, mode)
    except pxo.OracleError as e:
        a = px.Image.from_numpy(dst)
        with pytest.raises(px.PixieError, match=str(e)):
            a.draw_transform(px.Image.from_numpy(src), m, mode)
        return
    a = px.Image.from_numpy(dst)
    a.draw_transform(px.Image.from_numpy(src), m, mode)
    assert_same(a.to_numpy(), ref, f"{mat} mode {mode}")


@pytest.mark.parametrize("w,h", [(1, 1), (1, 7), (7, 1), (2, 2), (3, 5), (64, 64), (99, 99), (400, 177), (255, 3)])
@pytest.mark.parametrize("power", [0, 1, 2, 3])
def test_minify_by2(w, h, power):
    src = wl.premultiplied_image(w * 31 + h, w, h)
    ref = src.copy()
    for _ in range(power):
        ref = pxo.minify_by2(ref)
    out = px.Image.from_numpy(src).minify_by2(power)
    assert_same(out.to_numpy(), ref, f"{w}x{h} power {power}")


@pytest.mark.parametrize("w,h", [(1, 1), (3, 5), (33, 17)])
@pytest.mark.parametrize("power", [0, 1, 2])
def test_magnify_by2(w, h, power):
    src = wl.premultiplied_image(w * 7 + h, w, h)
    ref = src.copy()
    for _ in range(power):
        ref = pxo.magnify_by2(ref)
    out = px.Image.from_numpy(src).magnify_by2(power)
    assert_same(out.to_numpy(), ref, f"{w}x{h} power {power}")


def test_negative_power_errors():
    img = px.Image(4, 4)
    with pytest.raises(px.PixieError, match="Cannot minifyBy2 with negative power"):
        img.minify_by2(-1)
    with pytest.raises(px.PixieError, match="Cannot magnifyBy2 with negative power"):
        img.magnify_by2(-1)


def test_large_rotated_draw():
    """a 1024x1024 source rotated and scaled onto a 1536x1536 canvas"""
    dst, src = rand_case(123, 1536, 1536, 1024, 1024)
    mat = affine(33.0, 1.3, 0.9, 700.25, -100.5)
    gpu, ref = run_both(dst, src, mat, 0)
    assert_same(gpu, ref, "large")
