"""The C-ABI library loads without a GPU and exports every declared symbol."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pxg.h")
LIB = os.path.join(ROOT, "pixie_gb300", "libpxg.so")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pxg_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        from pixie_gb300 import build
        build.build()
    return ctypes.CDLL(LIB)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("pxg_image_fill_path", "pxg_image_stroke_path", "pxg_image_draw",
              "pxg_image_blur", "pxg_image_shadow", "pxg_take_error"):
        assert s in syms


def test_library_exports_every_declared_symbol(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_error_channel_without_gpu(lib):
    lib.pxg_take_error.restype = ctypes.c_char_p
    assert lib.pxg_check_error() == 0
    assert lib.pxg_take_error() == b""


def test_scene_recording_runs_on_the_host():
    """Recording a scene builds geometry on the host only (no GPU needed); a
    path raises at recording exactly when the oracle raises for it."""
    import pixie_gb300 as px
    from oracle import pxo
    from pixie_gb300 import workloads as wl
    items = wl.dense_scene(2, n_paths=200, size=256.0)
    sc = px.Scene()
    got, want = [], []
    img = pxo.new_image(256, 256)
    for i, it in enumerate(items):
        paint = px.Paint(it["color"], 1.0, it["blend"])
        try:
            if it["kind"] == "fill":
                sc.fill_path(it["cmds"], paint, None, it["winding"])
            else:
                sc.stroke_path(it["cmds"], paint, None, it["width"], it["cap"], it["join"], it["miter"])
        except px.PixieError as e:
            got.append((i, str(e)))
        try:
            if it["kind"] == "fill":
                pxo.fill_path(img, it["cmds"], it["color"], 1.0, it["blend"], None, it["winding"])
            else:
                pxo.stroke_path(img, it["cmds"], it["color"], 1.0, it["blend"], None, it["width"],
                                it["cap"], it["join"], it["miter"])
        except pxo.OracleError as e:
            want.append((i, str(e)))
    assert got == want and len(got) > 0
    assert len(sc) == len(items) - len(got)
    sc.clear()
    assert len(sc) == 0
    with pytest.raises(px.PixieError, match="Invalid line dash value"):
        sc.stroke_path("M 0 0 L 10 10", [1, 1, 1, 1], dashes=(1.0, 0.0))
    assert len(sc) == 0
