"""Path commands: pixie's ``Path`` object, its SVG parser and its builders.

A path is pixie's flat ``seq[float32]`` of ``[kind, params...]`` records
(src/pixie/paths.nim:18-27); ``kind`` is the float-encoded
``PathCommandKind`` ordinal.  This module mirrors the reference's path API
(paths.nim:68-652: ``parsePath``, ``moveTo``, ``lineTo``, ``bezierCurveTo``,
``quadraticCurveTo``, ``ellipticalArcTo``, ``arc``, ``arcTo``, ``rect``,
``roundedRect``, ``ellipse``, ``circle``, ``polygon``) with float32 arithmetic
(:mod:`pixie_gb300.f32`), so the command values equal the reference's.  The
commands are what the C ABI's fill/stroke entry points consume.
"""
from __future__ import annotations

import math

import numpy as np

from . import f32 as F

# PathCommandKind ordinals  paths.nim:18-22
CLOSE, MOVE, LINE, HLINE, VLINE, CUBIC, SCUBIC, QUAD, TQUAD, ARC = range(10)
RMOVE, RLINE, RHLINE, RVLINE, RCUBIC, RSCUBIC, RQUAD, RTQUAD, RARC = range(10, 19)

_PARAMS = {CLOSE: 0, MOVE: 2, LINE: 2, RMOVE: 2, RLINE: 2, TQUAD: 2, RTQUAD: 2,
           HLINE: 1, VLINE: 1, RHLINE: 1, RVLINE: 1, CUBIC: 6, RCUBIC: 6,
           SCUBIC: 4, RSCUBIC: 4, QUAD: 4, RQUAD: 4, ARC: 7, RARC: 7}


def parameter_count(kind: int) -> int:
    """paths.nim:72-81"""
    return _PARAMS[kind]


class PixieError(Exception):
    """The reference's PixieError (common.nim:4)."""


# Nim typing: a float32 meeting a float64 constant (PI, TAU, splineCircleK)
# is promoted to float64 and narrowed back to float32 where it is stored in a
# float32 (a command value, a Vec2 field).  Pinned by the polygon/arc goldens.
_SPLINE_CIRCLE_K = 4.0 * (-1.0 + 2.0 ** 0.5) / 3  # paths.nim:564 (float64)
_PI = 3.141592653589793
_TAU = 2.0 * _PI


class Path:
    """pixie's Path (paths.nim:24-27): float32 commands plus start/at."""

    def __init__(self):
        self.commands: list[float] = []
        self.start = (0.0, 0.0)
        self.at = (0.0, 0.0)

    def copy(self) -> "Path":
        p = Path()
        p.commands = list(self.commands)
        p.start, p.at = self.start, self.at
        return p

    def array(self) -> np.ndarray:
        return np.asarray(self.commands, dtype=np.float32)

    # -- builders  paths.nim:275-652 ------------------------------------
    def close_path(self):
        self.commands.append(float(CLOSE))
        self.at = self.start

    def move_to(self, x, y):
        x, y = F.f32(x), F.f32(y)
        self.commands += [float(MOVE), x, y]
        self.start = (x, y)
        self.at = self.start

    def line_to(self, x, y):
        x, y = F.f32(x), F.f32(y)
        self.commands += [float(LINE), x, y]
        self.at = (x, y)

    def bezier_curve_to(self, x1, y1, x2, y2, x3, y3):
        v = [F.f32(t) for t in (x1, y1, x2, y2, x3, y3)]
        self.commands += [float(CUBIC)] + v
        self.at = (v[4], v[5])

    def quadratic_curve_to(self, x1, y1, x2, y2):
        v = [F.f32(t) for t in (x1, y1, x2, y2)]
        self.commands += [float(QUAD)] + v
        self.at = (v[2], v[3])

    def elliptical_arc_to(self, rx, ry, rotation, large, sweep, x, y):
        v = [F.f32(rx), F.f32(ry), F.f32(rotation), 1.0 if large else 0.0,
             1.0 if sweep else 0.0, F.f32(x), F.f32(y)]
        self.commands += [float(ARC)] + v
        self.at = (v[5], v[6])

    def arc(self, x, y, r, a0, a1, ccw=False):
        """paths.nim:392-431"""
        x, y, r, a0, a1 = (F.f32(t) for t in (x, y, r, a0, a1))
        if r == 0:
            return
        if r < 0:
            raise PixieError("Invalid arc, negative radius: " + str(r))
        dx = F.mul(r, F.cos(a0))
        dy = F.mul(r, F.sin(a0))
        x0, y0 = F.add(x, dx), F.add(y, dy)
        cw = not ccw
        if len(self.commands) == 0:
            self.move_to(x0, y0)
        elif abs(F.sub(self.at[0], x0)) > F.EPSILON or abs(F.sub(self.at[1], y0)) > F.EPSILON:
            self.line_to(x0, y0)
        angle = F.sub(a0, a1) if ccw else F.sub(a1, a0)
        if angle < 0:
            angle = F.f32(math.fmod(angle, _TAU) + _TAU)
        if angle > _TAU - F.EPSILON:
            self.elliptical_arc_to(r, r, 0, True, cw, F.sub(x, dx), F.sub(y, dy))
            self.at = (x0, y0)
            self.elliptical_arc_to(r, r, 0, True, cw, x0, y0)
        elif angle > F.EPSILON:
            ax = F.add(x, F.mul(r, F.cos(a1)))
            ay = F.add(y, F.mul(r, F.sin(a1)))
            self.at = (ax, ay)
            self.elliptical_arc_to(r, r, 0, angle >= _PI, cw, ax, ay)

    def arc_to(self, x1, y1, x2, y2, r):
        """paths.nim:439-477"""
        x1, y1, x2, y2, r = (F.f32(t) for t in (x1, y1, x2, y2, r))
        if r < 0:
            raise PixieError("Invalid arc, negative radius: " + str(r))
        x0, y0 = self.at
        x21, y21 = F.sub(x2, x1), F.sub(y2, y1)
        x01, y01 = F.sub(x0, x1), F.sub(y0, y1)
        l01_2 = F.add(F.mul(x01, x01), F.mul(y01, y01))
        if len(self.commands) == 0:
            self.move_to(x0, y0)
        elif not (l01_2 > F.EPSILON):
            pass
        elif not (abs(F.sub(F.mul(y01, x21), F.mul(y21, x01))) > F.EPSILON) or r == 0:
            self.line_to(x1, y1)
        else:
            x20, y20 = F.sub(x2, x0), F.sub(y2, y0)
            l21_2 = F.add(F.mul(x21, x21), F.mul(y21, y21))
            l20_2 = F.add(F.mul(x20, x20), F.mul(y20, y20))
            l21 = F.sqrt(l21_2)
            l01 = F.sqrt(l01_2)
            cosang = F.div(F.sub(F.add(l21_2, l01_2), l20_2), F.mul(F.mul(2.0, l21), l01))
            # (PI - arccos(..)) / 2 is float64, so l, t01 and t21 are float64
            ll = r * math.tan((_PI - F.acos(cosang)) / 2)
            t01 = ll / l01
            t21 = ll / l21
            if abs(t01 - 1) > F.EPSILON:
                self.line_to(F.f32(x1 + t01 * x01), F.f32(y1 + t01 * y01))
            ax = F.f32(x1 + t21 * x21)
            ay = F.f32(y1 + t21 * y21)
            self.at = (ax, ay)
            self.elliptical_arc_to(r, r, 0, False, F.mul(y01, x20) > F.mul(x01, y20), ax, ay)

    def rect(self, x, y, w, h, clockwise=True):
        """paths.nim:484-499"""
        x, y, w, h = (F.f32(t) for t in (x, y, w, h))
        xw, yh = F.add(x, w), F.add(y, h)
        self.move_to(x, y)
        if clockwise:
            self.line_to(xw, y)
            self.line_to(xw, yh)
            self.line_to(x, yh)
        else:
            self.line_to(x, yh)
            self.line_to(xw, yh)
            self.line_to(xw, y)
        self.close_path()

    def rounded_rect(self, x, y, w, h, nw, ne, se, sw, clockwise=True):
        """paths.nim:515-595"""
        x, y, w, h, nw, ne, se, sw = (F.f32(t) for t in (x, y, w, h, nw, ne, se, sw))
        max_r = min(F.div(w, 2.0), F.div(h, 2.0))

        def clampr(v):
            v = v if v <= max_r else max_r
            return v if v >= 0 else 0.0

        nw, ne, se, sw = clampr(nw), clampr(ne), clampr(se), clampr(sw)
        if nw == 0 and ne == 0 and se == 0 and sw == 0:
            self.rect(x, y, w, h, clockwise)
            return
        s = _SPLINE_CIRCLE_K
        A, S, M = F.add, F.sub, F.mul
        t1 = (A(x, nw), y)
        t2 = (S(A(x, w), ne), y)
        r1 = (A(x, w), A(y, ne))
        r2 = (A(x, w), S(A(y, h), se))
        b1 = (S(A(x, w), se), A(y, h))
        b2 = (A(x, sw), A(y, h))
        l1 = (x, S(A(y, h), sw))
        l2 = (x, A(y, nw))
        # vec2(-nw * s, 0): the float64 product is narrowed into the Vec2
        t1h = (A(t1[0], F.f32(-nw * s)), t1[1])
        t2h = (A(t2[0], F.f32(ne * s)), t2[1])
        r1h = (r1[0], A(r1[1], F.f32(-ne * s)))
        r2h = (r2[0], A(r2[1], F.f32(se * s)))
        b1h = (A(b1[0], F.f32(se * s)), b1[1])
        b2h = (A(b2[0], F.f32(-sw * s)), b2[1])
        l1h = (l1[0], A(l1[1], F.f32(sw * s)))
        l2h = (l2[0], A(l2[1], F.f32(-nw * s)))
        if clockwise:
            self.move_to(*t1)
            self.line_to(*t2)
            self.bezier_curve_to(*t2h, *r1h, *r1)
            self.line_to(*r2)
            self.bezier_curve_to(*r2h, *b1h, *b1)
            self.line_to(*b2)
            self.bezier_curve_to(*b2h, *l1h, *l1)
            self.line_to(*l2)
            self.bezier_curve_to(*l2h, *t1h, *t1)
        else:
            self.move_to(*t1)
            self.bezier_curve_to(*t1h, *l2h, *l2)
            self.line_to(*l1)
            self.bezier_curve_to(*l1h, *b2h, *b2)
            self.line_to(*b1)
            self.bezier_curve_to(*b1h, *r2h, *r2)
            self.line_to(*r1)
            self.bezier_curve_to(*r1h, *t2h, *t2)
            self.line_to(*t1)
        self.close_path()

    def ellipse(self, cx, cy, rx, ry):
        """paths.nim:604-616"""
        cx, cy, rx, ry = (F.f32(t) for t in (cx, cy, rx, ry))
        mx, my = _SPLINE_CIRCLE_K * rx, _SPLINE_CIRCLE_K * ry  # float64
        A, S = F.add, F.sub
        self.move_to(A(cx, rx), cy)
        self.bezier_curve_to(A(cx, rx), cy + my, cx + mx, A(cy, ry), cx, A(cy, ry))
        self.bezier_curve_to(cx - mx, A(cy, ry), S(cx, rx), cy + my, S(cx, rx), cy)
        self.bezier_curve_to(S(cx, rx), cy - my, cx - mx, S(cy, ry), cx, S(cy, ry))
        self.bezier_curve_to(cx + mx, S(cy, ry), A(cx, rx), cy - my, A(cx, rx), cy)
        self.close_path()

    def circle(self, cx, cy, r):
        self.ellipse(cx, cy, r, r)

    def polygon(self, x, y, size, sides):
        """paths.nim:630-646"""
        if sides <= 2:
            raise PixieError("Invalid polygon sides value")
        x, y, size = F.f32(x), F.f32(y), F.f32(size)
        # sin/cos of float64 arguments: the vertices are float64 sums narrowed
        # by moveTo/lineTo.
        self.move_to(x + size * math.sin(0.0), y - size * math.cos(0.0))
        for side in range(1, sides):
            ang = float(side) * 2.0 * _PI / float(sides)
            self.line_to(x + size * math.sin(ang), y - size * math.cos(ang))
        self.close_path()


def parse_path(path: str) -> Path:
    """SVG path string -> commands, following parsePath (paths.nim:119-262)."""
    result = Path()
    if len(path) == 0:
        return result
    state = {"p": 0, "numberStart": 0, "armed": False, "hitDecimal": False, "kind": MOVE}
    numbers: list[float] = []

    def finish_number():
        ns = state["numberStart"]
        if ns > 0:
            try:
                numbers.append(F.f32(float(path[ns:state["p"]])))
            except ValueError:
                raise PixieError("Invalid path, parsing parameter failed")
        state["numberStart"] = 0
        state["hitDecimal"] = False

    def finish_command():
        finish_number()
        if state["armed"]:
            kind = state["kind"]
            pc = parameter_count(kind)
            if pc == 0:
                if len(numbers) != 0:
                    raise PixieError("Invalid path, unexpected parameters")
                result.commands.append(float(kind))
            else:
                if len(numbers) % pc != 0:
                    raise PixieError("Invalid path, wrong number of parameters")
                for batch in range(len(numbers) // pc):
                    if batch > 0:
                        if kind == MOVE:
                            kind = LINE
                        elif kind == RMOVE:
                            kind = RLINE
                    result.commands.append(float(kind))
                    result.commands.extend(numbers[batch * pc:(batch + 1) * pc])
                numbers.clear()
                state["kind"] = kind
        state["armed"] = True

    def expects_arc_flag():
        return state["kind"] in (ARC, RARC) and len(numbers) % 7 in (3, 4)

    letters = {"m": RMOVE, "l": RLINE, "h": RHLINE, "v": RVLINE, "c": RCUBIC, "s": RSCUBIC,
               "q": RQUAD, "t": RTQUAD, "a": RARC, "z": CLOSE, "M": MOVE, "L": LINE,
               "H": HLINE, "V": VLINE, "C": CUBIC, "S": SCUBIC, "Q": QUAD, "T": TQUAD,
               "A": ARC, "Z": CLOSE}
    while state["p"] < len(path):
        p = state["p"]
        ch = path[p]
        if ch in letters:
            finish_command()
            state["kind"] = letters[ch]
        elif ch in "-+":
            if state["numberStart"] > 0 and path[p - 1] in "eE":
                pass
            else:
                finish_number()
                state["numberStart"] = p
        elif ch == ".":
            if state["hitDecimal"] or expects_arc_flag():
                finish_number()
            state["hitDecimal"] = True
            if state["numberStart"] == 0:
                state["numberStart"] = p
        elif ch in " ,\r\n\t":
            finish_number()
        else:
            if state["numberStart"] > 0 and expects_arc_flag():
                finish_number()
            if p - 1 == state["numberStart"] and path[p - 1] == "0":
                finish_number()
            if state["numberStart"] == 0:
                state["numberStart"] = p
        state["p"] = p + 1
    finish_command()
    return result


def as_commands(path) -> np.ndarray:
    """A Path, an SVG path string, or a command array -> float32 commands."""
    if isinstance(path, str):
        return parse_path(path).array()
    if isinstance(path, Path):
        return path.array()
    return np.ascontiguousarray(path, dtype=np.float32)
