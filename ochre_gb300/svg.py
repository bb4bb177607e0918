"""SVG input: path data, a minimal document reader, and scene rendering.

The reference renders SVG files through usvg (examples/svg.rs:104-165),
which is not available here; this module reads the subset such files use:

* path data (SVG 1.1 §8.3): M/m L/l H/h V/v C/c S/s Q/q T/t A/a Z/z, implicit
  command repetition, number forms with exponents and without separators;
  elliptical arcs become conic segments (``PathCmd.Conic``, at most 90° each,
  weight cos(Δθ/2) — the rational-quadratic form of a circular arc mapped
  through the ellipse's affine frame);
* ``<path>``, ``<rect>``, ``<circle>``, ``<ellipse>``, ``<line>``,
  ``<polyline>``, ``<polygon>`` inside nested ``<g>`` elements, with
  ``transform`` (matrix / translate / scale / rotate / skewX / skewY),
  ``fill``, ``stroke``, ``stroke-width``, ``opacity``, ``fill-opacity``,
  ``stroke-opacity`` given as attributes or in ``style``; colours as
  ``#rgb``, ``#rrggbb``, ``rgb(r, g, b)`` or a few names.

Each painted path becomes one rasterizer: its fill (if any), then its stroke
(if any), exactly as the example does (one ``Rasterizer`` per paint,
examples/svg.rs:139-156).  Stroke widths are in the path's own space.
"""
from __future__ import annotations

import math
import re
import xml.etree.ElementTree as ET
from dataclasses import dataclass
from typing import List, Optional, Tuple

import numpy as np

from .batch import BatchBuilder
from .rasterizer import PathCmd, Vec2

_NUM = re.compile(r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?")
_ARGS = {"M": 2, "L": 2, "H": 1, "V": 1, "C": 6, "S": 4, "Q": 4, "T": 2, "A": 7, "Z": 0}


class _Scanner:
    """Character-level reader of path data (numbers may touch each other:
    "1-2.5.5e1"; arc flags are single digits that may touch: "0 011 1")."""

    def __init__(self, d: str):
        self.d = d
        self.i = 0

    def _skip(self):
        d, i = self.d, self.i
        while i < len(d) and d[i] in " \t\r\n,":
            i += 1
        self.i = i

    def command(self) -> Optional[str]:
        self._skip()
        if self.i < len(self.d) and self.d[self.i] in "MmLlHhVvCcSsQqTtAaZz":
            self.i += 1
            return self.d[self.i - 1]
        return None

    def done(self) -> bool:
        self._skip()
        return self.i >= len(self.d)

    def number(self) -> float:
        self._skip()
        m = _NUM.match(self.d, self.i)
        if not m:
            raise ValueError(f"expected a number at {self.d[self.i:self.i + 12]!r}")
        self.i = m.end()
        return float(m.group(0))

    def flag(self) -> bool:
        self._skip()
        if self.i < len(self.d) and self.d[self.i] in "01":
            self.i += 1
            return self.d[self.i - 1] == "1"
        raise ValueError(f"expected an arc flag at {self.d[self.i:self.i + 12]!r}")


def _arc_to_conics(x0, y0, rx, ry, phi_deg, large, sweep, x1, y1) -> List[PathCmd]:
    """SVG arc (endpoint form) as conic segments of at most 90 degrees
    (SVG 1.1 appendix F.6 for the centre form)."""
    if x0 == x1 and y0 == y1:
        return []
    rx, ry = abs(rx), abs(ry)
    if rx == 0.0 or ry == 0.0:
        return [PathCmd.Line(Vec2(x1, y1))]
    phi = math.radians(phi_deg % 360.0)
    cp, sp = math.cos(phi), math.sin(phi)
    dx, dy = (x0 - x1) / 2.0, (y0 - y1) / 2.0
    x1p, y1p = cp * dx + sp * dy, -sp * dx + cp * dy
    lam = (x1p * x1p) / (rx * rx) + (y1p * y1p) / (ry * ry)
    if lam > 1.0:
        s = math.sqrt(lam)
        rx, ry = rx * s, ry * s
    num = rx * rx * ry * ry - rx * rx * y1p * y1p - ry * ry * x1p * x1p
    den = rx * rx * y1p * y1p + ry * ry * x1p * x1p
    coef = math.sqrt(max(0.0, num / den)) if den > 0 else 0.0
    if large == sweep:
        coef = -coef
    cxp, cyp = coef * rx * y1p / ry, -coef * ry * x1p / rx
    cx = cp * cxp - sp * cyp + (x0 + x1) / 2.0
    cy = sp * cxp + cp * cyp + (y0 + y1) / 2.0

    def ang(ux, uy, vx, vy):
        a = math.atan2(ux * vy - uy * vx, ux * vx + uy * vy)
        return a

    th1 = ang(1.0, 0.0, (x1p - cxp) / rx, (y1p - cyp) / ry)
    dth = ang((x1p - cxp) / rx, (y1p - cyp) / ry, (-x1p - cxp) / rx, (-y1p - cyp) / ry)
    if not sweep and dth > 0:
        dth -= 2.0 * math.pi
    elif sweep and dth < 0:
        dth += 2.0 * math.pi
    n = max(1, int(math.ceil(abs(dth) / (math.pi / 2.0) - 1e-9)))
    step = dth / n
    out = []

    def pt(t):
        ex, ey = rx * math.cos(t), ry * math.sin(t)
        return cp * ex - sp * ey + cx, sp * ex + cp * ey + cy

    for k in range(n):
        a0, a1 = th1 + k * step, th1 + (k + 1) * step
        am = 0.5 * (a0 + a1)
        w = math.cos(step / 2.0)
        # control point: intersection of the tangents = point at the mid angle / cos(half step)
        ex, ey = rx * math.cos(am) / w, ry * math.sin(am) / w
        ctrl = (cp * ex - sp * ey + cx, sp * ex + cp * ey + cy)
        end = pt(a1) if k + 1 < n else (x1, y1)
        out.append(PathCmd.Conic(Vec2(*ctrl), Vec2(*end), w))
    return out


def parse_path(d: str) -> List[PathCmd]:
    """SVG path data -> PathCmd list (absolute coordinates)."""
    sc = _Scanner(d)
    out: List[PathCmd] = []
    cur = (0.0, 0.0)
    start = (0.0, 0.0)
    last_ctrl: Optional[Tuple[float, float]] = None   # for S (cubic) / T (quadratic)
    last_kind = None
    cmd = None
    # After a closepath the next drawing command starts a new subpath at the
    # same initial point (SVG 1.1 §8.3.3); ochre's Close moves nothing
    # (rasterizer.rs:154), so that subpath gets an explicit Move.
    after_close = False
    while not sc.done():
        c = sc.command()
        if c is not None:
            if cmd is None and c not in "Mm":
                raise ValueError("path data must start with a moveto")
            cmd = c
        elif cmd is None or cmd in "Zz":
            raise ValueError("path data must start with a command")
        if cmd in "Zz":
            out.append(PathCmd.Close())
            cur = start
            last_ctrl, last_kind = None, None
            after_close = True
            continue
        up = cmd.upper()
        rel = cmd.islower()
        if after_close and up != "M":
            out.append(PathCmd.Move(Vec2(*start)))
        after_close = False
        if up == "A":
            a = [sc.number(), sc.number(), sc.number(), sc.flag(), sc.flag(), sc.number(), sc.number()]
        else:
            a = [sc.number() for _ in range(_ARGS[up])]
        ox, oy = cur if rel else (0.0, 0.0)
        if up == "M":
            cur = (ox + a[0], oy + a[1])
            start = cur
            out.append(PathCmd.Move(Vec2(*cur)))
            cmd = "l" if rel else "L"      # further pairs are line-tos
            last_ctrl, last_kind = None, None
        elif up == "L":
            cur = (ox + a[0], oy + a[1])
            out.append(PathCmd.Line(Vec2(*cur)))
            last_ctrl, last_kind = None, None
        elif up == "H":
            cur = ((cur[0] if rel else 0.0) + a[0], cur[1])
            out.append(PathCmd.Line(Vec2(*cur)))
            last_ctrl, last_kind = None, None
        elif up == "V":
            cur = (cur[0], (cur[1] if rel else 0.0) + a[0])
            out.append(PathCmd.Line(Vec2(*cur)))
            last_ctrl, last_kind = None, None
        elif up == "C":
            c1 = (ox + a[0], oy + a[1])
            c2 = (ox + a[2], oy + a[3])
            cur = (ox + a[4], oy + a[5])
            out.append(PathCmd.Cubic(Vec2(*c1), Vec2(*c2), Vec2(*cur)))
            last_ctrl, last_kind = c2, "C"
        elif up == "S":
            c1 = (2 * cur[0] - last_ctrl[0], 2 * cur[1] - last_ctrl[1]) if last_kind == "C" else cur
            c2 = (ox + a[0], oy + a[1])
            cur = (ox + a[2], oy + a[3])
            out.append(PathCmd.Cubic(Vec2(*c1), Vec2(*c2), Vec2(*cur)))
            last_ctrl, last_kind = c2, "C"
        elif up == "Q":
            q = (ox + a[0], oy + a[1])
            cur = (ox + a[2], oy + a[3])
            out.append(PathCmd.Quadratic(Vec2(*q), Vec2(*cur)))
            last_ctrl, last_kind = q, "Q"
        elif up == "T":
            q = (2 * cur[0] - last_ctrl[0], 2 * cur[1] - last_ctrl[1]) if last_kind == "Q" else cur
            cur = (ox + a[0], oy + a[1])
            out.append(PathCmd.Quadratic(Vec2(*q), Vec2(*cur)))
            last_ctrl, last_kind = q, "Q"
        else:   # A
            end = (ox + a[5], oy + a[6])
            out.extend(_arc_to_conics(cur[0], cur[1], a[0], a[1], a[2], a[3], a[4], end[0], end[1]))
            cur = end
            last_ctrl, last_kind = None, None
    return out


# ---------------------------------------------------------------------------
# documents
# ---------------------------------------------------------------------------
_NAMED = {"black": (0, 0, 0), "white": (255, 255, 255), "red": (255, 0, 0), "green": (0, 128, 0),
          "blue": (0, 0, 255), "yellow": (255, 255, 0), "gray": (128, 128, 128), "grey": (128, 128, 128),
          "orange": (255, 165, 0), "purple": (128, 0, 128), "navy": (0, 0, 128), "teal": (0, 128, 128)}


def parse_color(s: Optional[str]):
    """RGB triple, or None for 'none' / missing."""
    if s is None:
        return None
    s = s.strip()
    if s in ("none", "transparent", ""):
        return None
    if s.startswith("#"):
        h = s[1:]
        if len(h) == 3:
            return tuple(int(c * 2, 16) for c in h)
        if len(h) == 6:
            return tuple(int(h[k:k + 2], 16) for k in (0, 2, 4))
        raise ValueError(f"bad colour {s!r}")
    m = re.fullmatch(r"rgb\(\s*([\d.]+)(%?)\s*,\s*([\d.]+)(%?)\s*,\s*([\d.]+)(%?)\s*\)", s)
    if m:
        vals = []
        for v, pct in ((m.group(1), m.group(2)), (m.group(3), m.group(4)), (m.group(5), m.group(6))):
            f = float(v) * (2.55 if pct else 1.0)
            vals.append(int(max(0, min(255, round(f)))))
        return tuple(vals)
    if s.lower() in _NAMED:
        return _NAMED[s.lower()]
    raise ValueError(f"unsupported colour {s!r}")


def parse_transform(s: Optional[str]) -> np.ndarray:
    """SVG transform list -> 3x3 affine matrix (float64)."""
    m = np.eye(3)
    if not s:
        return m
    for name, args in re.findall(r"(matrix|translate|scale|rotate|skewX|skewY)\s*\(([^)]*)\)", s):
        v = [float(x) for x in _NUM.findall(args)]
        t = np.eye(3)
        if name == "matrix":
            a, b, c, d, e, f = v
            t = np.array([[a, c, e], [b, d, f], [0, 0, 1.0]])
        elif name == "translate":
            t[0, 2] = v[0]
            t[1, 2] = v[1] if len(v) > 1 else 0.0
        elif name == "scale":
            t[0, 0] = v[0]
            t[1, 1] = v[1] if len(v) > 1 else v[0]
        elif name == "rotate":
            a = math.radians(v[0])
            r = np.array([[math.cos(a), -math.sin(a), 0], [math.sin(a), math.cos(a), 0], [0, 0, 1.0]])
            if len(v) == 3:
                tr, back = np.eye(3), np.eye(3)
                tr[:2, 2] = v[1], v[2]
                back[:2, 2] = -v[1], -v[2]
                r = tr @ r @ back
            t = r
        elif name == "skewX":
            t[0, 1] = math.tan(math.radians(v[0]))
        elif name == "skewY":
            t[1, 0] = math.tan(math.radians(v[0]))
        m = m @ t
    return m


def _style(el, inherited: dict) -> dict:
    """Inherited paint properties; a group's opacity multiplies into its
    descendants' (no layer compositing)."""
    st = dict(inherited)
    own = {}
    for k in ("fill", "stroke", "stroke-width", "opacity", "fill-opacity", "stroke-opacity"):
        if el.get(k) is not None:
            own[k] = el.get(k)
    for decl in (el.get("style") or "").split(";"):
        if ":" in decl:
            k, v = decl.split(":", 1)
            own[k.strip()] = v.strip()
    if "opacity" in own:
        own["opacity"] = str(float(st.get("opacity", 1.0)) * float(own["opacity"]))
    st.update(own)
    return st


def _shape_path(el) -> Optional[List[PathCmd]]:
    tag = el.tag.split("}")[-1]
    g = lambda k, dflt=0.0: float(el.get(k, dflt))
    if tag == "path":
        return parse_path(el.get("d", ""))
    if tag == "rect":
        x, y, w, h = g("x"), g("y"), g("width"), g("height")
        return [PathCmd.Move(Vec2(x, y)), PathCmd.Line(Vec2(x + w, y)), PathCmd.Line(Vec2(x + w, y + h)),
                PathCmd.Line(Vec2(x, y + h)), PathCmd.Close()]
    if tag in ("circle", "ellipse"):
        cx, cy = g("cx"), g("cy")
        rx = g("r") if tag == "circle" else g("rx")
        ry = g("r") if tag == "circle" else g("ry")
        return parse_path(f"M{cx + rx},{cy} A{rx},{ry} 0 0 1 {cx - rx},{cy} A{rx},{ry} 0 0 1 {cx + rx},{cy} Z")
    if tag == "line":
        return [PathCmd.Move(Vec2(g("x1"), g("y1"))), PathCmd.Line(Vec2(g("x2"), g("y2")))]
    if tag in ("polyline", "polygon"):
        v = [float(x) for x in _NUM.findall(el.get("points", ""))]
        pts = list(zip(v[0::2], v[1::2]))
        if not pts:
            return []
        out = [PathCmd.Move(Vec2(*pts[0]))] + [PathCmd.Line(Vec2(*p)) for p in pts[1:]]
        if tag == "polygon":
            out.append(PathCmd.Close())
        return out
    return None


@dataclass
class Paint:
    path: List[PathCmd]
    transform: np.ndarray            # 3x3
    rgba: Tuple[int, int, int, int]
    stroke_width: Optional[float]    # None: fill


def load_svg(text: str) -> Tuple[List[Paint], Tuple[float, float]]:
    """Painted paths of a document in drawing order, and its (width, height)."""
    root = ET.fromstring(text)
    size = (float(re.sub(r"[a-z%]+$", "", root.get("width", "0")) or 0),
            float(re.sub(r"[a-z%]+$", "", root.get("height", "0")) or 0))
    paints: List[Paint] = []

    def opacity(st, key):
        return float(st.get("opacity", 1.0)) * float(st.get(key, 1.0))

    def walk(el, m, st):
        tag = el.tag.split("}")[-1]
        m = m @ parse_transform(el.get("transform"))
        st = _style(el, st)
        if tag in ("defs", "clipPath", "mask", "symbol", "style", "title", "desc", "metadata"):
            return
        path = _shape_path(el)
        if path:
            fill = parse_color(st.get("fill", "black"))
            if fill is not None:
                a = int(round(255 * max(0.0, min(1.0, opacity(st, "fill-opacity")))))
                paints.append(Paint(path, m, (*fill, a), None))
            stroke = parse_color(st.get("stroke"))
            if stroke is not None:
                a = int(round(255 * max(0.0, min(1.0, opacity(st, "stroke-opacity")))))
                paints.append(Paint(path, m, (*stroke, a), float(st.get("stroke-width", 1.0))))
        for ch in el:
            walk(ch, m, st)

    walk(root, np.eye(3), {})
    return paints, size


def paints_to_batch(paints: List[Paint]):
    """One rasterizer per paint (examples/svg.rs:139-156); returns the batch
    and the RGBA8 colours [n, 4]."""
    from .rasterizer import encode_path
    bb = BatchBuilder()
    colors = np.zeros((len(paints), 4), np.uint8)
    for k, p in enumerate(paints):
        v, f = encode_path(p.path)
        m = p.transform
        xf = [m[0, 0], m[0, 1], m[1, 0], m[1, 1], m[0, 2], m[1, 2]]
        bb.begin_raster().fill(v, f, xf, stroke_width=p.stroke_width)
        colors[k] = p.rgba
    return bb.build(), colors


def render_svg(text: str, width: Optional[int] = None, height: Optional[int] = None, ctx=None,
               background=(255, 255, 255, 255)):
    """Rasterize and composite a document on the GPU; RGBA8 [h, w, 4] numpy."""
    import torch

    from .rasterizer import DeviceBatch, default_context
    paints, (w0, h0) = load_svg(text)
    w = int(width or w0 or 1)
    h = int(height or h0 or 1)
    ctx = ctx or default_context()
    canvas = torch.empty((h, w, 4), dtype=torch.uint8, device=f"cuda:{ctx.device}")
    canvas[:] = torch.tensor(background, dtype=torch.uint8)
    if paints:
        batch, colors = paints_to_batch(paints)
        r = ctx.rasterize_device(DeviceBatch(batch, ctx.device))
        ctx.composite(r, batch.n_rasters, torch.as_tensor(colors, device=canvas.device), canvas)
    torch.cuda.synchronize(ctx.device)
    return canvas.cpu().numpy()
