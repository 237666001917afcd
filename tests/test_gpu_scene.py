"""Dense scenes (many paths painted in order onto one canvas) through the
scene entry points, bit-exact against the oracle applying the same
fillPath/strokePath calls one after another."""
import numpy as np
import pytest

import pixie_gb300 as px
from oracle import pxo
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


def oracle_scene(items, w, h, bg=None, failed=None):
    """The reference's calls one after another; a call that raises (a few
    random arcs cannot be discretised by the reference's arc stepping) is
    skipped, as a caller catching PixieError per path would."""
    ref = pxo.new_image(w, h) if bg is None else bg.copy()
    for i, it in enumerate(items):
        try:
            if it["kind"] == "fill":
                pxo.fill_path(ref, it["cmds"], it["color"], it.get("opacity", 1.0), it["blend"],
                              it.get("mat"), it["winding"])
            else:
                pxo.stroke_path(ref, it["cmds"], it["color"], it.get("opacity", 1.0), it["blend"],
                                it.get("mat"), it["width"], it["cap"], it["join"], it["miter"],
                                it.get("dashes", ()))
        except pxo.OracleError as e:
            if failed is not None:
                failed.append((i, str(e)))
    return ref


def record_one(sc, it):
    paint = px.Paint(it["color"], it.get("opacity", 1.0), it["blend"])
    if it["kind"] == "fill":
        sc.fill_path(it["cmds"], paint, it.get("mat"), it["winding"])
    else:
        sc.stroke_path(it["cmds"], paint, it.get("mat"), it["width"], it["cap"], it["join"],
                       it["miter"], it.get("dashes", ()))


def record(items, failed=None):
    """Records the calls; a recording that raises is skipped (the same paths
    raise while the host builds their geometry as raise in the oracle)."""
    sc = px.Scene()
    for i, it in enumerate(items):
        try:
            record_one(sc, it)
        except px.PixieError as e:
            if failed is not None:
                failed.append((i, str(e)))
    return sc


@pytest.mark.parametrize("seed,n,size", [(1, 60, 128), (2, 200, 256), (3, 400, 512)])
def test_dense_scene_matches_sequential_oracle(seed, n, size):
    items = wl.dense_scene(seed, n_paths=n, size=float(size))
    f_ref, f_gpu = [], []
    ref = oracle_scene(items, size, size, failed=f_ref)
    sc = record(items, failed=f_gpu)
    assert f_gpu == f_ref
    assert len(sc) == n - len(f_ref)
    img = px.Image(size, size)
    img.draw_scene(sc)
    assert_same(img.to_numpy(), ref, f"scene seed {seed}")


def test_dense_scene_full_size_1024_2000_paths():
    items = wl.dense_scene(7, n_paths=2000, size=1024.0)
    f_ref, f_gpu = [], []
    ref = oracle_scene(items, 1024, 1024, failed=f_ref)
    sc = record(items, failed=f_gpu)
    assert f_gpu == f_ref
    img = px.Image(1024, 1024)
    img.draw_scene(sc)
    assert_same(img.to_numpy(), ref, "scene 1024^2 x 2000")


@pytest.mark.parametrize("threads", [1, 3, 0])
def test_batched_recording_equals_per_call_recording(threads):
    """record_batch builds the paths' geometry on host threads and appends
    them in order: the same scene, the same failures, the same bytes (with
    transforms and every blend mode)"""
    items = wl.dense_scene(5, n_paths=600, size=512.0)
    for k, it in enumerate(items):
        if k % 3 == 0:
            it["transform"] = [1.05, 0.02, 0, -0.03, 0.97, 0, 3.5, -2.25, 1]
        it["blend"] = k % 20
    f_one = []
    sc1 = px.Scene()
    for k, it in enumerate(items):
        paint = px.Paint(it["color"], 1.0, it["blend"])
        try:
            if it["kind"] == "fill":
                sc1.fill_path(it["cmds"], paint, it.get("transform"), it["winding"])
            else:
                sc1.stroke_path(it["cmds"], paint, it.get("transform"), it["width"], it["cap"], it["join"],
                                it["miter"])
            f_one.append(0)
        except px.PixieError:
            f_one.append(1)
    sc2 = px.Scene()
    status = sc2.record_batch(items, threads)
    assert list(status) == f_one
    assert len(sc1) == len(sc2)
    bg = wl.premultiplied_image(9, 512, 512)
    a = px.Image.from_numpy(bg)
    a.draw_scene(sc1)
    b = px.Image.from_numpy(bg)
    b.draw_scene(sc2)
    assert_same(b.to_numpy(), a.to_numpy(), f"batched recording, {threads} threads")


def test_scene_equals_one_call_per_path():
    items = wl.dense_scene(11, n_paths=150, size=300.0)
    a = px.Image(300, 300)
    a.draw_scene(record(items))
    b = px.Image(300, 300)
    for it in items:
        paint = px.Paint(it["color"], 1.0, it["blend"])
        try:
            if it["kind"] == "fill":
                b.fill_path(it["cmds"], paint, None, it["winding"])
            else:
                b.stroke_path(it["cmds"], paint, None, it["width"], it["cap"], it["join"], it["miter"])
        except px.PixieError:
            pass
    assert_same(a.to_numpy(), b.to_numpy(), "scene vs per-call")


def test_scene_on_background_with_every_mode_and_transforms():
    bg = wl.premultiplied_image(4, 320, 200)
    base = wl.dense_scene(13, n_paths=40, size=300.0)
    items = []
    for i, it in enumerate(base):
        it = dict(it)
        it["blend"] = i % 20  # includes MaskBlend (16), Overwrite, SubtractMask, ExcludeMask
        it["opacity"] = [1.0, 0.5, 0.25][i % 3]
        if i % 4 == 1:
            it["mat"] = np.array([0.8, 0.1, 0, -0.1, 0.7, 0, 15.5, -4.25, 1], np.float32)
        items.append(it)
    ref = oracle_scene(items, 320, 200, bg)
    img = px.Image.from_numpy(bg)
    img.draw_scene(record(items))
    assert_same(img.to_numpy(), ref, "scene with all modes")


def test_scene_rows_beyond_the_shared_scratch():
    # a comb with > 256 crossings per scanline: the scene kernel's wide path
    cmds = [1.0, 0.0, 0.0]
    for k in range(300):
        x = float(k * 3)
        cmds += [2.0, x + 1.5, 200.0, 2.0, x + 3.0, 0.0]
    cmds += [0.0]
    item = {"kind": "fill", "cmds": np.asarray(cmds, np.float32), "color": [0.2, 0.6, 0.3, 0.9],
            "blend": 0, "winding": 0}
    items = [item, dict(item, color=[0.9, 0.1, 0.1, 0.5], blend=2, winding=1)]
    ref = oracle_scene(items, 900, 200)
    img = px.Image(900, 200)
    img.draw_scene(record(items))
    assert_same(img.to_numpy(), ref, "wide scene rows")


def test_scene_error_stops_at_failing_path():
    # an empty path raises "Path int overflow detected" in fillShapes
    items = wl.dense_scene(17, n_paths=30, size=200.0)
    bad = np.zeros(0, np.float32)
    sc = record(items[:10])
    sc.fill_path(bad, px.Paint([1, 0, 0, 1]))
    for it in items[10:]:
        try:
            record_one(sc, it)
        except px.PixieError:
            pass
    ref = oracle_scene(items[:10], 200, 200)
    with pytest.raises(pxo.OracleError) as e:
        pxo.fill_path(ref.copy(), bad, [1, 0, 0, 1])
    img = px.Image(200, 200)
    with pytest.raises(px.PixieError) as g:
        img.draw_scene(sc)
    assert str(g.value) == str(e.value)
    assert_same(img.to_numpy(), ref, "paths before the failing one")


def test_scene_reuse_and_clear():
    items = wl.dense_scene(19, n_paths=25, size=128.0)
    sc = record(items)
    a = px.Image(128, 128)
    a.draw_scene(sc)
    a.draw_scene(sc)  # twice onto the same image
    ref = oracle_scene(items + items, 128, 128)
    assert_same(a.to_numpy(), ref, "scene drawn twice")
    sc.clear()
    assert len(sc) == 0
    b = px.Image(128, 128)
    b.draw_scene(sc)
    assert not b.to_numpy().any()


@pytest.mark.parametrize("slice_w", [1 << 20, 1024, 256, 64, 100, 32, 0])
def test_every_scene_configuration_writes_the_same_bytes(slice_w):
    items = wl.dense_scene(23, n_paths=120, size=300.0)
    ref = oracle_scene(items, 300, 300)
    sc = record(items)
    px.scene_config(slice_w)
    try:
        img = px.Image(300, 300)
        img.draw_scene(sc)
    finally:
        px.scene_config(256)
    assert_same(img.to_numpy(), ref, f"scene slice {slice_w}")


@pytest.mark.parametrize("cov_bytes", [0, 200000])
def test_scene_rows_recorded_as_spans_when_the_coverage_arena_is_small(cov_bytes):
    # 0: every row keeps its sample spans; 200 kB: some rows get coverage
    # bytes and the rest spans
    items = wl.dense_scene(29, n_paths=150, size=400.0)
    ref = oracle_scene(items, 400, 400)
    sc = record(items)
    px.scene_config(256, cov_bytes)
    try:
        img = px.Image(400, 400)
        img.draw_scene(sc)
    finally:
        px.scene_config(256, 64 << 20)
    assert_same(img.to_numpy(), ref, f"coverage arena {cov_bytes}")
