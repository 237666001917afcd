"""SVG front-end feeding the scene renderer: pixie's SVG loader
(src/pixie/fileformats/svg.nim) for documents of paths, lines, polylines,
polygons and rectangles with solid colours.

``parse_svg(text)`` restates ``parseSvg`` (svg.nim:37-330, :504-556): the
view box, the properties each element inherits from its groups (fill,
fill-rule, stroke, stroke-width, caps, joins, miter limit, dashes, opacity,
display, transform) and the element's path.  ``svg_items`` turns it into the
fillPath / strokePath calls ``newImage(svg)`` makes (svg.nim:557-600) -- the
first fill Overwrite, every later call Normal -- and ``svg_scene`` records them
into one :class:`pixie_gb300.Scene`, so a document is drawn with one setup and
one scene launch.  Gradients (``url(#...)`` fills) are not supported and raise.

Number parsing follows Nim: ``parseFloat`` gives a float64, stored in the
float32 fields; Mat3 products are vmath's column-major products in float32.
"""
from __future__ import annotations

import xml.etree.ElementTree as ET

import numpy as np

from . import f32 as F
from .paths import Path, PixieError, parse_path

IDENT = [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0]
DEFAULT_MITER = 4.0  # paths.nim:46 defaultMiterLimit
_CAPS = {"butt": 0, "round": 1, "square": 2}
_JOINS = {"miter": 0, "round": 1, "bevel": 2}
# CSS named colours (CSS Color Module) that documents use most; others raise
_NAMED = {"black": (0, 0, 0), "white": (255, 255, 255), "red": (255, 0, 0), "green": (0, 128, 0),
          "blue": (0, 0, 255), "yellow": (255, 255, 0), "gray": (128, 128, 128), "grey": (128, 128, 128),
          "navy": (0, 0, 128), "purple": (128, 0, 128), "pink": (255, 192, 203), "orange": (255, 165, 0),
          "silver": (192, 192, 192), "maroon": (128, 0, 0), "olive": (128, 128, 0), "lime": (0, 255, 0),
          "aqua": (0, 255, 255), "teal": (0, 128, 128), "fuchsia": (255, 0, 255), "cyan": (0, 255, 255),
          "magenta": (255, 0, 255)}


def _mat_mul(A, B):
    """vmath Mat3 * Mat3, column-major storage m[c * 3 + r], float32"""
    R = [0.0] * 9
    for c in range(3):
        for r in range(3):
            s = F.add(F.mul(A[0 * 3 + r], B[c * 3 + 0]), F.mul(A[1 * 3 + r], B[c * 3 + 1]))
            R[c * 3 + r] = F.add(s, F.mul(A[2 * 3 + r], B[c * 3 + 2]))
    return R


def _translate(x, y):
    return [1.0, 0.0, 0.0, 0.0, 1.0, 0.0, F.f32(x), F.f32(y), 1.0]


def _scale(x, y):
    return [F.f32(x), 0.0, 0.0, 0.0, F.f32(y), 0.0, 0.0, 0.0, 1.0]


def _rotate(angle):  # vmath rotate(angle: float32)
    c, s = F.cos(angle), F.sin(angle)
    return [c, s, 0.0, F.f32(-s), c, 0.0, 0.0, 0.0, 1.0]


def _float(s: str) -> float:
    try:
        return float(s)
    except ValueError:
        raise PixieError(f"Invalid SVG number {s!r}") from None


def _split_args(s: str):
    return [e for e in s.replace(",", " ").split(" ") if e]


def parse_color(s: str):
    """chroma's parseHtmlColor for hex colours and a few names -> straight
    float32 RGBA (each channel byte / 255)"""
    t = s.strip()
    if t.startswith("#"):
        h = t[1:]
        if len(h) == 3:
            rgb = [int(c * 2, 16) for c in h]
        elif len(h) == 6:
            rgb = [int(h[i:i + 2], 16) for i in (0, 2, 4)]
        else:
            raise PixieError(f"Invalid SVG color {s}")
    elif t.lower() in _NAMED:
        rgb = list(_NAMED[t.lower()])
    else:
        raise PixieError(f"Unsupported SVG color {s}")
    return [F.div(float(v), 255.0) for v in rgb] + [1.0]


class Props:
    """SvgProperties (svg.nim:19-30) with the defaults of initSvgProperties (:41-49)"""

    def __init__(self):
        self.display = True
        self.fill_rule = 0
        self.fill = "black"
        self.stroke = None  # straight RGBA, or None for rgbx(0, 0, 0, 0)
        self.stroke_width = 1.0
        self.cap = 0
        self.join = 0
        self.miter = DEFAULT_MITER
        self.dashes = []
        self.transform = list(IDENT)
        self.opacity = 1.0
        self.fill_opacity = 1.0
        self.stroke_opacity = 1.0

    def copy(self):
        p = Props.__new__(Props)
        p.__dict__.update(self.__dict__)
        p.dashes = list(self.dashes)
        p.transform = list(self.transform)
        return p


def _parse_props(node, inherited: Props) -> Props:  # svg.nim:51-286
    r = inherited.copy()
    a = {k: node.attrib.get(k, "") for k in (
        "fill-rule", "fill", "stroke", "stroke-width", "stroke-linecap", "stroke-linejoin", "stroke-miterlimit",
        "stroke-dasharray", "transform", "style", "display", "opacity", "fill-opacity", "stroke-opacity")}
    for pair in a["style"].split(";"):  # style never overrides an attribute
        parts = pair.split(":")
        if len(parts) == 2:
            k = parts[0].strip()
            key = {"fillOpacity": "fill-opacity", "strokeOpacity": "stroke-opacity"}.get(k, k)
            if key in a and key != "style" and key != "transform" and not a[key]:
                a[key] = parts[1].strip()
    if a["display"]:
        r.display = a["display"].strip() != "none"
    if a["opacity"]:
        r.opacity = F.f32(min(max(_float(a["opacity"]), 0.0), 1.0))
    if a["fill-rule"] == "nonzero":
        r.fill_rule = 0
    elif a["fill-rule"] == "evenodd":
        r.fill_rule = 1
    elif a["fill-rule"]:
        raise PixieError("Invalid fill-rule value " + a["fill-rule"])
    r.fill = inherited.fill if a["fill"] in ("", "currentColor") else a["fill"]
    st = a["stroke"]
    if st == "currentColor":
        if r.stroke is None:
            r.stroke = [0.0, 0.0, 0.0, 1.0]
    elif st == "none":
        r.stroke = None
    elif st:
        r.stroke = parse_color(st)
    if a["fill-opacity"]:
        r.fill_opacity = F.f32(min(max(_float(a["fill-opacity"]), 0.0), 1.0))
    if a["stroke-opacity"]:
        r.stroke_opacity = F.f32(min(max(_float(a["stroke-opacity"]), 0.0), 1.0))
    if a["stroke-width"]:
        sw = a["stroke-width"]
        if sw.endswith("px"):
            sw = sw[:-2]
        r.stroke_width = F.f32(_float(sw))
        if r.stroke is None:
            r.stroke = [0.0, 0.0, 0.0, 1.0]
    if a["stroke-linecap"] and a["stroke-linecap"] != "inherit":
        if a["stroke-linecap"] not in _CAPS:
            raise PixieError("Invalid stroke-linecap value " + a["stroke-linecap"])
        r.cap = _CAPS[a["stroke-linecap"]]
    if a["stroke-linejoin"] and a["stroke-linejoin"] != "inherit":
        if a["stroke-linejoin"] not in _JOINS:
            raise PixieError("Invalid stroke-linejoin value " + a["stroke-linejoin"])
        r.join = _JOINS[a["stroke-linejoin"]]
    if a["stroke-miterlimit"]:
        r.miter = F.f32(_float(a["stroke-miterlimit"]))
    if a["stroke-dasharray"]:
        r.dashes = r.dashes + [F.f32(_float(v)) for v in _split_args(a["stroke-dasharray"])]
    t = a["transform"]
    while t:
        i = t.find(")")
        if i == -1:
            raise PixieError("Unsupported SVG transform: " + a["transform"])
        f, t = t[:i + 1].strip(), t[i + 1:]
        if f.startswith("matrix("):
            v = _split_args(f[7:-1])
            if len(v) != 6:
                raise PixieError("Unsupported SVG transform: " + a["transform"])
            m = [F.f32(_float(v[0])), F.f32(_float(v[1])), 0.0, F.f32(_float(v[2])), F.f32(_float(v[3])), 0.0,
                 F.f32(_float(v[4])), F.f32(_float(v[5])), 1.0]
            r.transform = _mat_mul(r.transform, m)
        elif f.startswith("translate("):
            v = _split_args(f[10:-1])
            r.transform = _mat_mul(r.transform, _translate(_float(v[0]), _float(v[1]) if len(v) > 1 else 0.0))
        elif f.startswith("rotate("):
            v = _split_args(f[7:-1])
            angle = F.f32(_float(v[0]) * 3.141592653589793 / 180)
            cx = F.f32(_float(v[1])) if len(v) > 1 else 0.0
            cy = F.f32(_float(v[2])) if len(v) > 2 else 0.0
            m = _mat_mul(_mat_mul(_translate(cx, cy), _rotate(angle)), _translate(-cx, -cy))
            r.transform = _mat_mul(r.transform, m)
        elif f.startswith("scale("):
            v = _split_args(f[6:-1])
            sx = F.f32(_float(v[0]))
            sy = F.f32(_float(v[1])) if len(v) > 1 else sx
            r.transform = _mat_mul(r.transform, _scale(sx, sy))
        else:
            raise PixieError("Unsupported SVG transform: " + a["transform"])
    return r


def _tag(node):
    return node.tag.rsplit("}", 1)[-1]


def _elements(node, stack, out):  # parseSvgElement  svg.nim:288-502
    tag = _tag(node)
    if tag in ("title", "desc", "defs"):
        return
    if tag == "g":
        stack.append(_parse_props(node, stack[-1]))
        for child in node:
            _elements(child, stack, out)
        stack.pop()
        return
    props = _parse_props(node, stack[-1])
    attr = node.attrib.get
    if tag == "path":
        out.append((parse_path(attr("d", "")), props))
    elif tag == "line":
        p = Path()
        p.move_to(_float(attr("x1", "0")), _float(attr("y1", "0")))
        p.line_to(_float(attr("x2", "0")), _float(attr("y2", "0")))
        out.append((p, props))
    elif tag in ("polyline", "polygon"):
        pts = attr("points", "")
        vecs = []
        if "," in pts:
            for pair in pts.split(" "):
                parts = pair.split(",")
                if len(parts) != 2:
                    raise PixieError("Invalid SVG data")
                vecs.append((_float(parts[0]), _float(parts[1])))
        else:
            v = pts.split(" ")
            if len(v) % 2:
                raise PixieError("Invalid SVG data")
            vecs = [(_float(v[2 * i]), _float(v[2 * i + 1])) for i in range(len(v) // 2)]
        if not vecs:
            raise PixieError("Invalid SVG data")
        p = Path()
        p.move_to(*vecs[0])
        for v in vecs[1:]:
            p.line_to(*v)
        if tag == "polygon":
            p.close_path()
        out.append((p, props))
    elif tag == "rect":
        x, y = F.f32(_float(attr("x", "0"))), F.f32(_float(attr("y", "0")))
        w, h = F.f32(_float(attr("width", "0"))), F.f32(_float(attr("height", "0")))
        if w == 0 or h == 0:
            return
        rx = F.f32(max(_float(attr("rx", "0")), 0.0))
        ry = F.f32(max(_float(attr("ry", "0")), 0.0))
        p = Path()
        if rx > 0 or ry > 0:
            if rx == 0:
                rx = ry
            elif ry == 0:
                ry = rx
            rx = min(rx, F.div(w, 2.0))
            ry = min(ry, F.div(h, 2.0))
            p.move_to(F.add(x, rx), y)
            p.line_to(F.sub(F.add(x, w), rx), y)
            p.elliptical_arc_to(rx, ry, 0.0, False, True, F.add(x, w), F.add(y, ry))
            p.line_to(F.add(x, w), F.sub(F.add(y, h), ry))
            p.elliptical_arc_to(rx, ry, 0.0, False, True, F.sub(F.add(x, w), rx), F.add(y, h))
            p.line_to(F.add(x, rx), F.add(y, h))
            p.elliptical_arc_to(rx, ry, 0.0, False, True, x, F.sub(F.add(y, h), ry))
            p.line_to(x, F.add(y, ry))
            p.elliptical_arc_to(rx, ry, 0.0, False, True, F.add(x, rx), y)
        else:
            p.rect(x, y, w, h)
        out.append((p, props))
    elif tag in ("circle", "ellipse"):
        cx, cy = F.f32(_float(attr("cx", "0"))), F.f32(_float(attr("cy", "0")))
        if tag == "circle":
            rx = ry = F.f32(_float(attr("r", "")))
        else:
            rx, ry = F.f32(_float(attr("rx", "0"))), F.f32(_float(attr("ry", "0")))
        p = Path()
        p.ellipse(cx, cy, rx, ry)
        out.append((p, props))
    else:
        raise PixieError(f"Unsupported SVG tag: {tag}")


class Svg:
    def __init__(self, width: int, height: int, elements):
        self.width, self.height, self.elements = width, height, elements


def parse_svg(text: str, width: int = 0, height: int = 0) -> Svg:
    """parseSvg  svg.nim:504-566"""
    try:
        root = ET.fromstring(text)
    except ET.ParseError as e:
        raise PixieError("Invalid SVG data") from e
    if _tag(root) != "svg":
        raise PixieError("Invalid SVG data")
    vb = root.attrib.get("viewBox", "").split(" ")
    try:
        vx, vy, vw, vh = (int(v) for v in vb[:4])
    except ValueError:
        raise PixieError("Invalid SVG data") from None
    props = _parse_props(root, Props())
    if vx != 0 or vy != 0:
        props.transform = _mat_mul(props.transform, _translate(-vx, -vy))
    if width == 0 and height == 0:
        width, height = vw, vh
    else:
        props.transform = _mat_mul(props.transform, _scale(F.div(float(width), float(vw)),
                                                           F.div(float(height), float(vh))))
    stack = [props]
    out = []
    for node in root:
        _elements(node, stack, out)
    return Svg(width, height, out)


_PARAMS = {0: 0, 1: 2, 2: 2, 3: 1, 4: 1, 5: 6, 6: 4, 7: 4, 8: 2, 9: 7, 10: 2, 11: 2, 12: 1, 13: 1, 14: 6, 15: 4,
           16: 4, 17: 2, 18: 7}


def _draws(cmds) -> bool:
    """whether the command stream has a command other than Move / RMove / Close"""
    i, n = 0, len(cmds)
    while i < n:
        k = int(cmds[i])
        if k not in (0, 1, 10):
            return True
        i += 1 + _PARAMS.get(k, 0)
    return False


def svg_items(svg: Svg):
    """The fillPath / strokePath calls of newImage(svg)  svg.nim:568-600, as
    scene items (see Scene.record_batch): the first fill Overwrite, the rest
    Normal."""
    items = []
    blend = 17  # OverwriteBlend
    for path, p in svg.elements:
        if not (p.display and p.opacity > 0):
            continue
        cmds = path.array() if isinstance(path, Path) else np.asarray(path, np.float32)
        if not _draws(cmds):
            # a path of moves and closes only ("M x,y z"): the reference's
            # fillShapes raises on its empty bounds and newImage stops there;
            # this front-end leaves it out so the rest of the document renders
            continue
        if p.fill != "none":
            if p.fill.startswith("url("):
                raise PixieError("Unsupported SVG fill " + p.fill)
            items.append({"kind": "fill", "cmds": cmds, "color": parse_color(p.fill),
                          "opacity": F.mul(p.fill_opacity, p.opacity), "blend": blend,
                          "transform": p.transform, "winding": p.fill_rule})
        blend = 0  # NormalBlend
        if p.stroke is not None and p.stroke_width > 0:
            col = list(p.stroke)
            col[3] = F.mul(col[3], F.mul(p.opacity, p.stroke_opacity))
            items.append({"kind": "stroke", "cmds": cmds, "color": col, "opacity": 1.0, "blend": blend,
                          "transform": p.transform, "width": p.stroke_width, "cap": p.cap, "join": p.join,
                          "miter": p.miter, "dashes": list(p.dashes)})
    return items


def svg_scene(svg: Svg, threads: int = 0):
    """The document's calls recorded into one Scene (batched recording on host
    threads; a dashed stroke is recorded with its own call, which carries the
    dashes).  Returns (scene, per-call status)."""
    from . import Paint, Scene
    sc = Scene()
    items = svg_items(svg)
    status = []
    batch = []

    def flush():
        if batch:
            status.extend(int(v) for v in sc.record_batch(batch, threads))
            batch.clear()

    for it in items:
        if it["kind"] == "stroke" and it["dashes"]:
            flush()
            try:
                sc.stroke_path(it["cmds"], Paint(it["color"], it["opacity"], it["blend"]), it["transform"],
                               it["width"], it["cap"], it["join"], it["miter"], it["dashes"])
                status.append(0)
            except PixieError:
                status.append(1)
        else:
            batch.append(it)
    flush()
    return sc, np.asarray(status, np.int32)


def new_image(svg: Svg):
    """newImage(svg)  svg.nim:568-600: a transparent image of the document's
    size with every call drawn in order (one scene draw)."""
    from . import Image
    img = Image(svg.width, svg.height)
    sc, _ = svg_scene(svg)
    img.draw_scene(sc)
    return img
