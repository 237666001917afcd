"""Mask batches (many glyph-like paths, each into its own 8-bit mask, in one
graph launch) and their ordered composite onto a page, bit-exact against the
oracle: fillPath(color(1, 1, 1, 1)) onto a transparent image of the mask's
size, then draw(page, glyph, translate(x, y), mode) in batch order."""
import numpy as np
import pytest

import pixie_gb300 as px
from oracle import pxo
from pixie_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

WHITE = [1.0, 1.0, 1.0, 1.0]


def assert_same(gpu, cpu, what=""):
    gpu = np.asarray(gpu).astype(np.int32)
    cpu = np.asarray(cpu).astype(np.int32)
    assert gpu.shape == cpu.shape
    d = np.abs(gpu - cpu)
    n = int((d.reshape(d.shape[0], -1) > 0).sum()) if d.ndim == 2 else int((d.reshape(-1, 4).max(axis=1) > 0).sum())
    assert n == 0, f"{what}: max|delta|={int(d.max())} differing px={n}"


@pytest.fixture(scope="module", autouse=True)
def _init():
    px.lib().pxg_init(0)
    pxo.set_golden_mode(False)


def oracle_glyph(cmds, w, h, winding):
    img = pxo.new_image(w, h)
    pxo.fill_path(img, cmds, WHITE, 1.0, 0, None, winding)
    return img


def make_batch(glyphs):
    m = px.Masks()
    for cmds, w, h, wind in glyphs:
        m.add_path(cmds, w, h, None, wind)
    return m


def test_masks_match_oracle_alpha():
    glyphs, _ = wl.glyph_batch(3, n=200)
    m = make_batch(glyphs)
    m.render()
    for i, (cmds, w, h, wind) in enumerate(glyphs):
        ref = oracle_glyph(cmds, w, h, wind)
        # an image filled with white keeps four equal channels
        assert (ref[..., 0] == ref[..., 3]).all()
        assert_same(m.mask(i), ref[..., 3], f"mask {i}")


@pytest.mark.parametrize("threads", [1, 5, 0])
def test_batched_glyph_recording_equals_per_call(threads):
    """add_paths builds the glyphs' geometry on host threads and appends
    them in order: the same masks as one add_path per glyph, and a failing
    glyph adds none"""
    glyphs, _ = wl.glyph_batch(4, n=300)
    a = make_batch(glyphs)
    b = px.Masks()
    b.add_paths(glyphs, threads)
    a.render()
    b.render()
    for i in range(len(glyphs)):
        assert_same(b.mask(i), a.mask(i), f"mask {i}")
    c = px.Masks()
    bad = list(glyphs[:5]) + [(glyphs[5][0], 0, 10, 0)] + list(glyphs[6:10])
    with pytest.raises(px.PixieError, match="Image width and height must be > 0"):
        c.add_paths(bad, threads)
    assert len(c._sizes) == 0


@pytest.mark.parametrize("variant,rpi", [(0, 1), (1, 1), (1, 2), (1, 4), (0, 3)])
def test_every_row_configuration_writes_the_same_masks(variant, rpi):
    glyphs, _ = wl.glyph_batch(5, n=120)
    m = make_batch(glyphs)
    m.render_config(variant, rpi)
    for i, (cmds, w, h, wind) in enumerate(glyphs):
        assert_same(m.mask(i), oracle_glyph(cmds, w, h, wind)[..., 3], f"mask {i} cfg {variant},{rpi}")


def test_graph_replay_and_recapture():
    glyphs, _ = wl.glyph_batch(9, n=64)
    m = make_batch(glyphs)
    m.render()
    m.render()  # replays the captured launch
    m.render()
    first = [m.mask(i).copy() for i in range(len(glyphs))]
    extra, w, h, wind = wl.glyph(12345)
    m.add_path(extra, w, h, None, wind)  # a new shape: captured again
    m.render()
    for i, (cmds, gw, gh, gwind) in enumerate(glyphs):
        assert_same(m.mask(i), first[i], f"replayed mask {i}")
    assert_same(m.mask(len(glyphs)), oracle_glyph(extra, w, h, wind)[..., 3], "added mask")
    assert "mask_rows" in px.autotune_report()


def oracle_page(glyphs, pos, page, mode=0):
    ref = page.copy()
    for (cmds, w, h, wind), (x, y) in zip(glyphs, pos):
        g = oracle_glyph(cmds, w, h, wind)
        pxo.draw(ref, g, int(x), int(y), mode)
    return ref


@pytest.mark.parametrize("mode", [0, 2, 10, 17, 18, 19])
def test_draw_masks_in_order_matches_oracle(mode):
    glyphs, pos = wl.glyph_batch(4, n=300, page=700)
    pos = pos - 40  # some masks start left of / above the page
    bg = wl.premultiplied_image(8, 700, 650)
    ref = oracle_page(glyphs, pos, bg, mode)
    m = make_batch(glyphs)
    m.render()
    page = px.Image.from_numpy(bg)
    page.draw_masks(m, pos, mode)
    assert_same(page.to_numpy(), ref, f"page mode {mode}")


def test_draw_masks_rejects_maskblend():
    glyphs, pos = wl.glyph_batch(4, n=3, page=100)
    m = make_batch(glyphs)
    m.render()
    page = px.Image(100, 100)
    with pytest.raises(px.PixieError, match="MaskBlend"):
        page.draw_masks(m, pos, px.BlendMode.MaskBlend)


def test_glyph_batch_full_size_4096_on_4096_page():
    glyphs, pos = wl.glyph_batch(7, n=4096, page=4096)
    m = make_batch(glyphs)
    m.render()
    page = px.Image(4096, 4096)
    page.draw_masks(m, pos)
    ref = oracle_page(glyphs, pos, pxo.new_image(4096, 4096))
    assert_same(page.to_numpy(), ref, "4096 glyphs on 4096^2")
    for i in range(0, 4096, 97):
        cmds, w, h, wind = glyphs[i]
        assert_same(m.mask(i), oracle_glyph(cmds, w, h, wind)[..., 3], f"mask {i}")
