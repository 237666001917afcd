"""Parity at the full sizes of the composite-and-blur and serving workloads.

* draw of a 2048x2048 premultiplied RGBX image onto another under each of the
  16 blend modes and 4 mask modes (images.nim:468-529 blendRect);
* blur of a 4096x4096 image at radius 1, 4, 16 and 64 (images.nim:304-365),
  which runs the small-radius passes (r <= 8) and the tensor-core ring passes;
* render jobs at serving scale (canvas side >= 2048, >= 2000 dense-scene
  paths, one job blurred), served together by the continuous-batching server.

Every byte must equal the oracle's.  The oracle's blurs run in threads and
its scenes in row windows (oracle.pxo.draw_items), so the file finishes in
minutes on the host cores.
"""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

import pixie_gb300 as px
from oracle import pxo
from pixie_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
THREADS = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module", autouse=True)
def _init():
    px.lib().pxg_init(0)
    pxo.set_golden_mode(False)


def assert_same(gpu, cpu, what):
    d = np.abs(np.asarray(gpu).astype(np.int32) - np.asarray(cpu).astype(np.int32))
    n = int((d.reshape(-1, 4).max(axis=1) > 0).sum())
    assert n == 0, f"{what}: max|delta|={int(d.max())} differing px={n}"


def test_draw_2048_every_mode():
    a = wl.premultiplied_image(10, 2048, 2048)
    b = wl.premultiplied_image(15, 2048, 2048)
    B = px.Image.from_numpy(b)
    refs = {}

    def oracle_draw(mode):
        r = a.copy()
        pxo.draw(r, b, 0, 0, mode)
        return mode, r

    with ThreadPoolExecutor(THREADS) as ex:
        refs = dict(ex.map(oracle_draw, range(20)))
    for mode in range(20):
        A = px.Image.from_numpy(a)
        A.draw(B, (0, 0), mode)
        assert_same(A.to_numpy(), refs[mode], f"draw 2048^2 mode {mode} ({pxo.BLEND_MODES[mode]})")


def test_draw_2048_offset_every_mode():
    """the same images at a translation that is not a multiple of 4 pixels
    (the kernel's scalar path) and overhangs two edges"""
    a = wl.premultiplied_image(11, 2048, 2048)
    b = wl.premultiplied_image(16, 2048, 2048)
    B = px.Image.from_numpy(b)

    def oracle_draw(mode):
        r = a.copy()
        pxo.draw(r, b, 37, -501, mode)
        return mode, r

    with ThreadPoolExecutor(THREADS) as ex:
        refs = dict(ex.map(oracle_draw, range(20)))
    for mode in range(20):
        A = px.Image.from_numpy(a)
        A.draw(B, (37, -501), mode)
        assert_same(A.to_numpy(), refs[mode], f"draw 2048^2 at (37,-501) mode {mode}")


def test_blur_4096_radii():
    src = wl.premultiplied_image(19, 4096, 4096)

    def oracle_blur(r):
        x = src.copy()
        pxo.blur(x, r)
        return r, x

    with ThreadPoolExecutor(4) as ex:
        refs = dict(ex.map(oracle_blur, (1, 4, 16, 64)))
    for r in (1, 4, 16, 64):
        img = px.Image.from_numpy(src)
        img.blur(r)
        assert_same(img.to_numpy(), refs[r], f"blur 4096^2 r={r}")


def _record(items):
    sc = px.Scene()
    status = sc.record_batch(items, 0)
    return sc, int(np.asarray(status).sum())


def test_served_jobs_at_serving_scale():
    jobs = [{"side": 2048, "items": wl.dense_scene(501, n_paths=2000, size=2048.0), "blur": 0},
            {"side": 2048, "items": wl.dense_scene(502, n_paths=2000, size=2048.0), "blur": 12},
            {"side": 2304, "items": wl.dense_scene(503, n_paths=2200, size=2304.0), "blur": 0}]
    scenes = [_record(j["items"]) for j in jobs]
    sv = px.Server(40 << 30, 512, 16384)
    ids = {sv.submit(sc, j["side"], j["side"], j["blur"]): k for k, (j, (sc, _)) in enumerate(zip(jobs, scenes))}
    out = {}
    guard = 0
    while sv.pending() > 0:
        sv.step()
        for jid in sv.poll():
            out[ids[jid]] = sv.take(jid)[0]
        guard += 1
        assert guard < 100000
    for jid in sv.poll():
        out[ids[jid]] = sv.take(jid)[0]
    assert sv.stats()["peak_admitted"] == 3  # the three jobs were on the GPU together
    for k, j in enumerate(jobs):
        ref = pxo.new_image(j["side"], j["side"])
        skipped = pxo.draw_items(ref, j["items"], THREADS)
        assert skipped == scenes[k][1], f"job {k}: {skipped} paths raise in the oracle, {scenes[k][1]} on record"
        if j["blur"]:
            pxo.blur(ref, j["blur"])
        assert_same(out[k], ref, f"served job {k} ({j['side']}^2, {len(j['items'])} paths, blur {j['blur']})")


def test_dense_scene_full_size():
    """The dense-scene workload at its full size: 2000 mixed paths (30 %
    stroked, outlined on the GPU) painted in order onto 1024x1024."""
    items = wl.dense_scene(7, n_paths=2000, size=1024.0)
    sc, failed = _record(items)
    img = px.Image(1024, 1024)
    img.draw_scene(sc)
    ref = pxo.new_image(1024, 1024)
    skipped = pxo.draw_items(ref, items, THREADS)
    assert skipped == failed
    assert_same(img.to_numpy(), ref, "dense scene 1024^2, 2000 paths")
