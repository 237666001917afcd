"""Seeded synthetic inputs for the five measurement workloads.

All randomness is splitmix64 -> float32 via ``(u >> 40) * 2**-24 * range``,
so the CPU oracle and the GPU see identical float32 inputs.
  plain fill   one 512x512 image, one closed path of 64 random cubics
  composite    2048x2048 premultiplied RGBX images (alpha U{0..255},
               RGB U{0..alpha}); blur of a 4096x4096 image; shadow of a
               1024x1024 mask of 64 discs
  dense scene  2000 mixed line/quad/cubic/arc paths on a 1024x1024 canvas
  glyph batch  4096 glyph-like outlines, bbox 8..256 px, 10..120 quads,
               1..4 contours (inner ones reversed)
"""
from __future__ import annotations

import math

import numpy as np

from .paths import Path

_M64 = (1 << 64) - 1


def splitmix64(seed: int, n: int) -> np.ndarray:
    """n consecutive outputs of splitmix64 starting from `seed`."""
    with np.errstate(over="ignore"):
        idx = np.arange(1, n + 1, dtype=np.uint64)
        z = np.uint64(seed & _M64) + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))


def uniform01(seed: int, n: int) -> np.ndarray:
    """float32 uniform in [0, 1) with 24 random bits."""
    u = splitmix64(seed, n) >> np.uint64(40)
    return (u.astype(np.float32) * np.float32(2.0 ** -24)).astype(np.float32)


def uniform(seed: int, n: int, lo: float, hi: float) -> np.ndarray:
    return (np.float32(lo) + uniform01(seed, n) * np.float32(hi - lo)).astype(np.float32)


def randint(seed: int, n: int, lo: int, hi: int) -> np.ndarray:
    """Integers uniform in [lo, hi]."""
    u = splitmix64(seed, n)
    return (lo + (u % np.uint64(hi - lo + 1)).astype(np.int64)).astype(np.int64)


# -- plain fill -----------------------------------------------------------------
PLAIN_COLOR = [np.float32(v) / np.float32(255) for v in (252, 66, 123, 255)]


def plain_path(seed: int, n_cubics: int = 64, size: float = 512.0) -> np.ndarray:
    """Move + n cubics + Close, every point uniform in [0, size)^2."""
    v = uniform(seed * 7919 + 1, 2 + 6 * n_cubics, 0.0, size)
    cmds = [1.0, float(v[0]), float(v[1])]
    for i in range(n_cubics):
        cmds.append(5.0)
        cmds.extend(float(t) for t in v[2 + 6 * i:8 + 6 * i])
    cmds.append(0.0)
    return np.asarray(cmds, np.float32)


# -- composite ------------------------------------------------------------------
def premultiplied_image(seed: int, w: int, h: int) -> np.ndarray:
    """alpha uniform in {0..255}, each RGB uniform in {0..alpha}."""
    n = w * h
    u = splitmix64(seed * 104729 + 3, 4 * n).reshape(n, 4)
    a = (u[:, 3] % np.uint64(256)).astype(np.uint32)
    img = np.empty((n, 4), np.uint8)
    img[:, 3] = a
    for c in range(3):
        img[:, c] = (u[:, c] % (a.astype(np.uint64) + np.uint64(1))).astype(np.uint8)
    return img.reshape(h, w, 4)


def disc_mask_path(seed: int, n: int = 64, size: float = 1024.0) -> np.ndarray:
    """64 discs (centre U[0,size)^2, radius U[4,128]) as one path."""
    c = uniform(seed * 31 + 5, 2 * n, 0.0, size)
    r = uniform(seed * 31 + 6, n, 4.0, 128.0)
    p = Path()
    for i in range(n):
        p.circle(float(c[2 * i]), float(c[2 * i + 1]), float(r[i]))
    return p.array()


# -- dense scene ----------------------------------------------------------------
def dense_scene(seed: int, n_paths: int = 2000, size: float = 1024.0):
    """Paths of 4..60 commands mixing line/quad/cubic/arc; 70% filled (half
    NonZero, half EvenOdd, alpha U[64,255]), 30% stroked (width log-U
    [0.5, 8], cap/join uniform, miter limit 4); blend uniform over 16 modes."""
    out = []
    for i in range(n_paths):
        s = seed * 1000003 + i * 17
        ncmd = int(randint(s, 1, 4, 60)[0])
        kinds = randint(s + 1, ncmd, 0, 3)
        pts = uniform(s + 2, 6 * ncmd + 2, 0.0, size)
        arc = uniform(s + 3, 4 * ncmd, 0.0, 1.0)
        cmds = [1.0, float(pts[0]), float(pts[1])]
        for k in range(ncmd):
            p = pts[2 + 6 * k:8 + 6 * k]
            if kinds[k] == 0:
                cmds += [2.0, float(p[0]), float(p[1])]
            elif kinds[k] == 1:
                cmds += [7.0, float(p[0]), float(p[1]), float(p[2]), float(p[3])]
            elif kinds[k] == 2:
                cmds += [5.0] + [float(t) for t in p]
            else:
                a = arc[4 * k:4 * k + 4]
                rx = float(np.float32(4.0 * math.exp(float(a[0]) * math.log(128.0))))
                ry = float(np.float32(4.0 * math.exp(float(a[1]) * math.log(128.0))))
                rot = float(np.float32(a[2] * 360.0))
                flags = int(a[3] * 4)
                cmds += [9.0, rx, ry, rot, float(flags & 1), float((flags >> 1) & 1),
                         float(p[0]), float(p[1])]
        attr = uniform(s + 4, 8, 0.0, 1.0)
        filled = attr[0] < 0.7
        col = [float(attr[1]), float(attr[2]), float(attr[3]),
               float(np.float32((64 + attr[4] * 191.0) / 255.0))]
        blend = int(attr[5] * 16) % 16
        item = {"cmds": np.asarray(cmds, np.float32), "color": col, "blend": blend}
        if filled:
            cmds.append(0.0)
            item["cmds"] = np.asarray(cmds, np.float32)
            item.update(kind="fill", winding=int(attr[6] < 0.5))
        else:
            w = float(np.float32(0.5 * math.exp(float(attr[6]) * math.log(16.0))))
            item.update(kind="stroke", width=w, cap=int(attr[7] * 3) % 3,
                        join=int(attr[2] * 3) % 3, miter=4.0)
        out.append(item)
    return out


# -- glyph batch ----------------------------------------------------------------
def glyph(seed: int):
    """One glyph-like outline: returns (commands, width, height, winding)."""
    a = uniform(seed * 7 + 11, 8, 0.0, 1.0)
    side = float(8.0 * math.exp(float(a[0]) * math.log(32.0)))
    w = max(1, int(side))
    h = max(1, int(side * (0.7 + 0.6 * float(a[1]))))
    n_contours = 1 + int(a[2] * 4) % 4
    total_q = 10 + int(a[3] * 111)
    per = max(3, total_q // n_contours)
    p = Path()
    jit = uniform(seed * 7 + 12, 2 * per * n_contours, -0.08, 0.08)
    for c in range(n_contours):
        scale_c = 1.0 - 0.22 * c
        cx, cy = w / 2.0, h / 2.0
        rx, ry = 0.45 * w * scale_c, 0.45 * h * scale_c
        pts = []
        for k in range(per):
            t = 2 * math.pi * k / per
            jx = float(jit[2 * (c * per + k)])
            jy = float(jit[2 * (c * per + k) + 1])
            pts.append((cx + rx * (1 + jx) * math.cos(t), cy + ry * (1 + jy) * math.sin(t)))
        if c % 2 == 1:
            pts.reverse()
        # quadratic outline through midpoints, controls at the jittered points
        mids = [((pts[k][0] + pts[(k + 1) % per][0]) / 2, (pts[k][1] + pts[(k + 1) % per][1]) / 2)
                for k in range(per)]
        p.move_to(*mids[-1])
        for k in range(per):
            p.quadratic_curve_to(pts[k][0], pts[k][1], mids[k][0], mids[k][1])
        p.close_path()
    winding = int(a[4] < 0.5)
    return p.array(), w, h, winding


def glyph_batch(seed: int, n: int = 4096, page: int = 4096):
    glyphs = [glyph(seed * 100003 + i) for i in range(n)]
    pos = randint(seed * 13 + 1, 2 * n, 0, page - 1).reshape(n, 2)
    return glyphs, pos


# -- serving ----------------------------------------------------------------------
def serving_job(seed: int, min_side: int = 256, max_side: int = 4096, min_paths: int = 10,
                max_paths: int = 5000, blur_share: float = 0.2):
    """One render job: canvas side log-uniform in [min_side, max_side], a dense
    scene of min_paths..max_paths paths over the canvas, and on blur_share of
    jobs a blur of radius uniform in {2..32}."""
    a = uniform(seed * 2654435761 + 17, 4, 0.0, 1.0)
    side = int(min_side * math.exp(float(a[0]) * math.log(max_side / min_side)))
    n = min_paths + int(float(a[1]) * (max_paths - min_paths + 1))
    n = min(n, max_paths)
    blur = 2 + int(float(a[2]) * 31) if float(a[3]) < blur_share else 0
    return {"side": side, "items": dense_scene(seed, n_paths=n, size=float(side)), "blur": blur}


def poisson_arrivals(seed: int, rate: float, n: int) -> np.ndarray:
    """n arrival times (seconds from 0) of a Poisson process of `rate` jobs/s."""
    u = uniform01(seed * 7 + 3, n).astype(np.float64)
    return np.cumsum(-np.log1p(-u) / rate)


def heart_commands(scale: float = 1.0):
    """pixie's test heart (tests/test_paints.nim:3-9, a 100x100 design) scaled by `scale`."""
    from .paths import parse_path
    k = float(scale)
    return parse_path(f"""
        M {10 * k},{30 * k}
        A {20 * k},{20 * k} 0,0,1 {50 * k},{30 * k}
        A {20 * k},{20 * k} 0,0,1 {90 * k},{30 * k}
        Q {90 * k},{60 * k} {50 * k},{90 * k}
        Q {10 * k},{60 * k} {10 * k},{30 * k} z
    """).array()
