"""Bit-exact parity of the CUDA library (through the C ABI) with the oracle.

Every comparison is on premultiplied RGBX bytes; a mismatch is reported as
max |delta| in 8-bit units and the number of differing pixels, and both must
be 0.  The oracle is the scalar (-d:pixieNoSimd) restatement in
oracle/pxo.cpp, itself pinned to the reference's golden PNGs
(tests/test_oracle_goldens.py).
"""
import math

import numpy as np
import pytest

import pixie_gb300 as px
from cases import CASES
from gpu_backend import GpuBackend
from oracle import pxo
from oracle_backend import OracleBackend
from pixie_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def assert_same(gpu, cpu, what=""):
    gpu = np.asarray(gpu).astype(np.int32)
    cpu = np.asarray(cpu).astype(np.int32)
    assert gpu.shape == cpu.shape
    d = np.abs(gpu - cpu)
    n = int((d.reshape(-1, 4).max(axis=1) > 0).sum())
    assert n == 0, f"{what}: max|delta|={int(d.max())} differing px={n}"


@pytest.fixture(scope="module", autouse=True)
def _init():
    px.lib().pxg_init(0)
    pxo.set_golden_mode(False)


# -- the reference's golden scenes ---------------------------------------------
@pytest.mark.parametrize("name", sorted(CASES))
def test_golden_scene_matches_oracle(name):
    fn = CASES[name][0]
    g = GpuBackend()
    assert_same(g.pixels(fn(g)), fn(OracleBackend()), name)


def test_golden_known_answers_on_gpu():
    from cases import fill_optimization_pixel, mask_out_of_bounds_transparent
    assert fill_optimization_pixel(GpuBackend()) == (255, 128, 64, 255)
    assert mask_out_of_bounds_transparent(GpuBackend())


# -- fill: random paths ------------------------------------------------------------
@pytest.mark.parametrize("seed", list(range(1, 13)))
def test_plain_fill_512_random_cubics(seed):
    cmds = wl.plain_path(seed)
    ref = pxo.new_image(512, 512)
    pxo.fill_path(ref, cmds, wl.PLAIN_COLOR)
    img = px.Image(512, 512)
    img.fill_path(cmds, wl.PLAIN_COLOR)
    assert_same(img.to_numpy(), ref, f"seed {seed}")


@pytest.mark.parametrize("blend", list(range(20)))
@pytest.mark.parametrize("winding", [0, 1])
def test_fill_every_mode_on_random_backdrop(blend, winding):
    seed = 100 + blend * 2 + winding
    bg = wl.premultiplied_image(seed, 160, 120)
    cmds = wl.plain_path(seed, n_cubics=9, size=170.0)
    color = [0.8, 0.3, 0.6, 0.7]
    ref = bg.copy()
    pxo.fill_path(ref, cmds, color, 0.9, blend, None, winding)
    img = px.Image.from_numpy(bg)
    img.fill_path(cmds, px.Paint(color, 0.9, blend), None, winding)
    assert_same(img.to_numpy(), ref, f"blend {blend} winding {winding}")


@pytest.mark.parametrize("seed", [3, 4])
def test_fill_transform_and_relative_commands(seed):
    p = px.parse_path("m 20 20 l 60 5 q 30 40 -10 70 t -30 10 c -10 -20 5 -40 -20 -60 z "
                      "M 120 30 h 50 v 60 s -30 20 -50 -10 Z a 20 10 30 1 0 40 20")
    mat = [np.float32(v) for v in (0.9, 0.2, 0, -0.3, 1.1, 0, 13.5, 7.25, 1)]
    bg = wl.premultiplied_image(seed, 230, 170)
    for winding in (0, 1):
        ref = bg.copy()
        pxo.fill_path(ref, p.array(), [0.2, 0.9, 0.4, 1.0], 1.0, 0, mat, winding)
        img = px.Image.from_numpy(bg)
        img.fill_path(p, [0.2, 0.9, 0.4, 1.0], mat, winding)
        assert_same(img.to_numpy(), ref, f"winding {winding}")


def test_fill_paths_outside_and_across_edges():
    paths = ["M -20 -20 L 50 10 L 10 60 Z", "M 150 150 L 250 180 L 190 260 Z",
             "M -30.5 10.25 L 40.75 10.25 L 40.75 50.5 L -30.5 50.5 Z",
             "M 10 -50 L 60 -50 L 60 -10 L 10 -10 Z", "M 95.5 5 L 300 5 L 300 95.5 L 95.5 95.5 Z"]
    for blend in (0, 16, 17, 18, 19, 2):
        for s in paths:
            bg = wl.premultiplied_image(7, 100, 100)
            cmds = px.parse_path(s).array()
            ref = bg.copy()
            pxo.fill_path(ref, cmds, [1, 0.5, 0.25, 0.75], 1.0, blend)
            img = px.Image.from_numpy(bg)
            img.fill_path(cmds, px.Paint([1, 0.5, 0.25, 0.75], 1.0, blend))
            assert_same(img.to_numpy(), ref, f"{s} blend {blend}")


def test_dense_scene_slice():
    scene = wl.dense_scene(5, n_paths=120, size=256.0)
    ref = pxo.new_image(256, 256)
    img = px.Image(256, 256)
    for it in scene:
        if it["kind"] == "fill":
            pxo.fill_path(ref, it["cmds"], it["color"], 1.0, it["blend"], None, it["winding"])
            img.fill_path(it["cmds"], px.Paint(it["color"], 1.0, it["blend"]), None, it["winding"])
        else:
            pxo.stroke_path(ref, it["cmds"], it["color"], 1.0, it["blend"], None, it["width"],
                            it["cap"], it["join"], it["miter"])
            img.stroke_path(it["cmds"], px.Paint(it["color"], 1.0, it["blend"]), None, it["width"],
                            it["cap"], it["join"], it["miter"])
    assert_same(img.to_numpy(), ref, "dense scene")


@pytest.mark.parametrize("cap,join", [(0, 0), (1, 1), (2, 2), (0, 2), (2, 0)])
def test_strokes_with_dashes(cap, join):
    p = px.parse_path("M 10 10 L 80 30 L 40 90 Q 90 90 110 20 C 130 0 150 80 180 60")
    bg = wl.premultiplied_image(11, 200, 110)
    for dashes in ((), (6.0, 3.0), (2.0, 5.0, 9.0)):
        ref = bg.copy()
        pxo.stroke_path(ref, p.array(), [0.1, 0.4, 0.9, 0.8], 1.0, 0, None, 5.5, cap, join, 4.0, dashes)
        img = px.Image.from_numpy(bg)
        img.stroke_path(p, [0.1, 0.4, 0.9, 0.8], None, 5.5, cap, join, 4.0, dashes)
        assert_same(img.to_numpy(), ref, f"dashes {dashes}")


def test_batch_matches_single_calls():
    glyphs, _ = wl.glyph_batch(3, n=48)
    imgs = [px.Image(w, h) for (_, w, h, _) in glyphs]
    status = px.fill_paths_batch(imgs, [g[0] for g in glyphs], [[1, 1, 1, 1]] * len(glyphs),
                                 winding_rules=[g[3] for g in glyphs])
    assert (status == 0).all()
    for (cmds, w, h, wind), im in zip(glyphs, imgs):
        ref = pxo.new_image(w, h)
        pxo.fill_path(ref, cmds, [1, 1, 1, 1], 1.0, 0, None, wind)
        assert_same(im.to_numpy(), ref, "glyph")


# -- blend modes, draw ---------------------------------------------------------------
def test_blend_modes_exhaustive_sample():
    n = 1 << 18
    bd = wl.premultiplied_image(21, 512, 512).reshape(-1, 4)[:n]
    src = wl.premultiplied_image(22, 512, 512).reshape(-1, 4)[:n]
    B = px.Image.from_numpy(bd.reshape(512, -1, 4))
    S = px.Image.from_numpy(src.reshape(512, -1, 4))
    O = px.Image(512, 512)
    for mode in range(20):
        px.blend_pixels(mode, B.device_ptr, S.device_ptr, O.device_ptr, n)
        assert_same(O.to_numpy().reshape(-1, 4)[:n], pxo.blend_pixels(mode, bd, src), f"mode {mode}")


@pytest.mark.parametrize("mode", list(range(20)))
def test_draw_every_mode(mode):
    a = wl.premultiplied_image(31 + mode, 300, 200)
    b = wl.premultiplied_image(61 + mode, 164, 120)
    for tx, ty in ((0, 0), (40, 24), (-13, 7), (250, 150), (-200, 0), (301, 5), (17, -119)):
        ref = a.copy()
        pxo.draw(ref, b, tx, ty, mode)
        A = px.Image.from_numpy(a)
        A.draw(px.Image.from_numpy(b), (tx, ty), mode)
        assert_same(A.to_numpy(), ref, f"mode {mode} at {tx},{ty}")


# -- blur / spread / shadow -----------------------------------------------------------
@pytest.mark.parametrize("radius", [1, 4, 16, 64, 2.6])
def test_blur(radius):
    img = wl.premultiplied_image(41, 230, 157)
    for oob in ((0, 0, 0, 0), (10, 20, 30, 200)):
        color = [np.float32(v) / np.float32(255) for v in oob]  # a straight Color
        ref = img.copy()
        pxo.blur(ref, radius, pxo.color_to_rgbx(color))  # asRgbx premultiplies it
        G = px.Image.from_numpy(img)
        G.blur(radius, color)
        assert_same(G.to_numpy(), ref, f"radius {radius} oob {oob}")


def test_blur_large_radius_direct_path():
    img = wl.premultiplied_image(42, 97, 1203)
    ref = img.copy()
    pxo.blur(ref, 700)
    G = px.Image.from_numpy(img)
    G.blur(700)
    assert_same(G.to_numpy(), ref, "radius 700")


@pytest.mark.parametrize("s", [4, -3, 1])
def test_spread(s):
    img = wl.premultiplied_image(43, 211, 99)
    ref = img.copy()
    pxo.spread(ref, s)
    G = px.Image.from_numpy(img)
    G.spread(s)
    assert_same(G.to_numpy(), ref, f"spread {s}")


def test_shadow():
    mask = pxo.new_image(256, 256)
    pxo.fill_path(mask, wl.disc_mask_path(9, n=12, size=256.0), [1, 1, 1, 1])
    col = [0.0, 0.0, 0.0, 1.0]
    for off, sp, bl in (((8, 8), 4, 12), ((0, 0), 0, 3), ((-5, 3), -2, 0)):
        ref = pxo.shadow(mask, off[0], off[1], sp, bl, col)
        out = px.Image.from_numpy(mask).shadow(off, sp, bl, col)
        assert_same(out.to_numpy(), ref, f"shadow {off} {sp} {bl}")


# -- errors ------------------------------------------------------------------------------
def test_errors_match_reference_messages():
    img = px.Image(20, 20)
    with pytest.raises(px.PixieError, match="Cannot apply negative blur"):
        img.blur(-3)
    with pytest.raises(px.PixieError, match="Path int overflow detected"):
        img.fill_path(np.zeros(0, np.float32), [1, 1, 1, 1])
    with pytest.raises(px.PixieError, match="Invalid line dash value"):
        img.stroke_path("M 0 0 L 10 10", [1, 1, 1, 1], dashes=(1.0, 0.0))
    with pytest.raises(px.PixieError, match="Image width and height must be > 0"):
        px.Image(0, 5)
    # the context stays usable after errors
    img.fill_path("M 2 2 L 18 2 L 18 18 Z", [1, 0, 0, 1])
    assert img.to_numpy()[10, 15, 3] > 0
