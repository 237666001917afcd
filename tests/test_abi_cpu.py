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
