"""Second, independent CPU restatement of ochre 0.2.0's rasterizer in numpy
float32 scalar arithmetic (test infrastructure: used only to cross-check the C
oracle on small inputs).  Structured differently from oracle/ochre_oracle.c on
purpose: it first produces the full line list (path.rs flatten + rasterizer.rs
implicit closes), then walks every line (rasterizer.rs:72-140), then bins with
a dictionary keyed by tile (rasterizer.rs:185-268).

Every float operation is an explicit np.float32 operation in the reference's
evaluation order; Rust's ``f32::min``/``max`` return the non-NaN operand.
"""
from __future__ import annotations

import math

import numpy as np

F = np.float32
ONE = F(1.0)
ZERO = F(0.0)
TOL = F(0.1)


def rmin(a, b):
    if a != a:
        return b
    if b != b:
        return a
    return a if a < b else b


def rmax(a, b):
    if a != a:
        return b
    if b != b:
        return a
    return a if a > b else b


def as_i16(v):
    v = float(v)
    if v != v:
        return 0
    if v <= -32768.0:
        return -32768
    if v >= 32767.0:
        return 32767
    return int(v)  # truncation toward zero


def as_u8(v):
    v = float(v)
    if v != v or v <= 0.0:
        return 0
    if v >= 255.0:
        return 255
    return int(v)


def wrap16(v):
    return ((int(v) + 32768) & 0xFFFF) - 32768


def fdiv8(v):
    return v // 8  # Python floor division == div_euclid for divisor 8


def signum16(v):
    v = float(v)
    if v != v:
        return 0
    return -1 if math.copysign(1.0, v) < 0 else 1


def lerp(t, a, b):
    return ((ONE - t) * a[0] + t * b[0], (ONE - t) * a[1] + t * b[1])


def length(v):
    return np.sqrt(v[0] * v[0] + v[1] * v[1])


def apply(xf, p):
    x = xf[0] * p[0] + xf[1] * p[1]
    y = xf[2] * p[0] + xf[3] * p[1]
    return (x + xf[4], y + xf[5])


def lines_of_raster(commands):
    """commands: list of (verb, [points as float32 pairs], weight) already in
    device space.  Returns the ordered list of line_to targets paired with
    their start points, i.e. every line_to call the reference makes."""
    first = (ZERO, ZERO)
    last = (ZERO, ZERO)
    out = []

    def line_to(p):
        nonlocal last
        out.append((last, p))
        last = p

    def move_to(p):
        nonlocal first, last
        if not (last[0] == first[0] and last[1] == first[1]):
            line_to(first)
        first = p
        last = p
        out.append(("move", p))

    for verb, pts, w in commands:
        l0 = last
        if verb == 0:
            move_to(pts[0])
        elif verb == 1:
            line_to(pts[0])
        elif verb == 2:
            c, p = pts
            v = (l0[0] - F(2.0) * c[0] + p[0], l0[1] - F(2.0) * c[1] + p[1])
            dt = np.sqrt((F(4.0) * TOL) / length(v))
            t = ZERO
            while t < ONE:
                t = rmin(t + dt, ONE)
                line_to(lerp(t, lerp(t, l0, c), lerp(t, c, p)))
        elif verb == 3:
            c1, c2, p = pts
            a = tuple(F(-1.0) * l0[i] + F(3.0) * c1[i] - F(3.0) * c2[i] + p[i] for i in range(2))
            b = tuple(F(3.0) * (l0[i] - F(2.0) * c1[i] + c2[i]) for i in range(2))
            conc = rmax(length(b), length((a[0] + b[0], a[1] + b[1])))
            dt = np.sqrt((np.sqrt(F(8.0)) * TOL) / conc)
            t = ZERO
            while t < ONE:
                t = rmin(t + dt, ONE)
                p01, p12, p23 = lerp(t, l0, c1), lerp(t, c1, c2), lerp(t, c2, p)
                line_to(lerp(t, lerp(t, p01, p12), lerp(t, p12, p23)))
        elif verb == 4:
            c, p = pts
            wc = (w * c[0], w * c[1])

            def rec(t0, t1, p0, p1):
                t = F(0.5) * (t0 + t1)
                p01 = lerp(t, l0, wc)
                p12 = lerp(t, wc, p)
                denom = (ONE - t) * (ONE - t) + F(2.0) * t * (ONE - t) * w + t * t
                q = lerp(t, p01, p12)
                mid = ((ONE / denom) * q[0], (ONE / denom) * q[1])
                e = (mid[0] - F(0.5) * (p0[0] + p1[0]), mid[1] - F(0.5) * (p0[1] + p1[1]))
                if length(e) > TOL:
                    rec(t0, t, p0, mid)
                    rec(t, t1, mid, p1)
                else:
                    line_to(mid)
                    line_to(p1)

            rec(ZERO, ONE, l0, p)
    if not (last[0] == first[0] and last[1] == first[1]):
        line_to(first)
    return out


def walk(a, p, tile_y_prev, incs, tincs):
    """rasterizer.rs:73-137 for one line; returns the new tile_y_prev."""
    if a[0] == p[0] and a[1] == p[1]:
        return tile_y_prev
    x_dir, y_dir = signum16(p[0] - a[0]), signum16(p[1] - a[1])
    dtdx = ONE / (p[0] - a[0])
    dtdy = ONE / (p[1] - a[1])
    x, y = as_i16(np.floor(a[0])), as_i16(np.floor(a[1]))
    row_t0 = col_t0 = ZERO
    if a[1] == p[1]:
        row_t1 = F(np.inf)
    else:
        ny = F(wrap16(y + 1)) if p[1] > a[1] else F(y)
        row_t1 = rmin(dtdy * (ny - a[1]), ONE)
    if a[0] == p[0]:
        col_t1 = F(np.inf)
    else:
        nx = F(wrap16(x + 1)) if p[0] > a[0] else F(x)
        col_t1 = rmin(dtdx * (nx - a[0]), ONE)
    xs, ys = abs(dtdx), abs(dtdy)
    while True:
        t0 = rmax(row_t0, col_t0)
        t1 = rmin(row_t1, col_t1)
        p0 = lerp(t0, a, p)
        p1 = lerp(t1, a, p)
        h = p1[1] - p0[1]
        right = F(wrap16(x + 1))
        area = F(0.5) * h * ((right - p0[0]) + (right - p1[0]))
        incs.append((x, y, area, h))
        if row_t1 < col_t1:
            row_t0 = row_t1
            row_t1 = rmin(row_t1 + ys, ONE)
            y = wrap16(y + y_dir)
        else:
            col_t0 = col_t1
            col_t1 = rmin(col_t1 + xs, ONE)
            x = wrap16(x + x_dir)
        end = row_t0 == ONE or col_t0 == ONE
        if end:
            x, y = as_i16(np.floor(p[0])), as_i16(np.floor(p[1]))
        ty = fdiv8(y)
        if ty != tile_y_prev:
            sign = ((ty - tile_y_prev + 128) & 0xFF) - 128
            tincs.append((fdiv8(x), min(tile_y_prev, ty), sign))
            tile_y_prev = ty
        if end:
            return tile_y_prev


def rasterize(commands):
    """Returns (tiles, spans, n_increments): tiles = [(x, y, bytes64)],
    spans = [(x, y, w, index of preceding tile)]."""
    incs, tincs = [], []
    tile_y_prev = 0
    for item in lines_of_raster(commands):
        if item[0] == "move":
            tile_y_prev = fdiv8(as_i16(np.floor(item[1][1])))
            continue
        tile_y_prev = walk(item[0], item[1], tile_y_prev, incs, tincs)
    # accumulate per tile in increment order (any order is a valid outcome
    # of the reference's unstable sort)
    acc = {}
    for x, y, area, h in incs:
        key = (fdiv8(y), fdiv8(x))
        cell = (y & 7) * 8 + (x & 7)
        a, hh = acc.setdefault(key, ([ZERO] * 64, [ZERO] * 64))
        a[cell] = a[cell] + area
        hh[cell] = hh[cell] + h
    if not incs:
        acc[(0, 0)] = ([ZERO] * 64, [ZERO] * 64)
    keys = sorted(acc)
    tincs.sort(key=lambda t: (t[1], t[0]))
    tiles, spans = [], []
    prev = [ZERO] * 8
    ti = 0
    winding = 0
    for i, (ty, tx) in enumerate(keys):
        areas, heights = acc[(ty, tx)]
        data = bytearray(64)
        nxt = [ZERO] * 8
        for yy in range(8):
            s = prev[yy]
            for xx in range(8):
                data[yy * 8 + xx] = as_u8(rmin(abs(s + areas[yy * 8 + xx]) * F(256.0), F(255.0)))
                s = s + heights[yy * 8 + xx]
            nxt[yy] = s
        tiles.append((wrap16(tx * 8), wrap16(ty * 8), bytes(data)))
        same_row = i + 1 < len(keys) and keys[i + 1][0] == ty
        prev = nxt if same_row else [ZERO] * 8
        if same_row and keys[i + 1][1] > tx + 1:
            while ti < len(tincs) and (tincs[ti][1], tincs[ti][0]) <= (ty, tx):
                winding += tincs[ti][2]
                ti += 1
            if winding != 0:
                w = (keys[i + 1][1] - tx - 1) * 8 & 0xFFFF
                spans.append((wrap16((tx + 1) * 8), wrap16(ty * 8), w, len(tiles) - 1))
    return tiles, spans, len(incs)


def path_polyline(verbs, flo):
    """path.rs:113-142 (flatten) on raw float32 points: list of (verb, point)."""
    from ochre_gb300.batch import FLOATS_PER_VERB
    last = (ZERO, ZERO)
    out = []
    o = 0
    for v in verbs:
        v = int(v)
        fl = [F(q) for q in flo[o:o + int(FLOATS_PER_VERB[v])]]
        o += int(FLOATS_PER_VERB[v])
        if v in (0, 1):
            out.append((v, (fl[0], fl[1])))
            last = (fl[0], fl[1])
        elif v == 5:
            out.append((5, None))
        else:
            npts = {2: 2, 3: 3, 4: 2}[v]
            pts = [(fl[2 * k], fl[2 * k + 1]) for k in range(npts)]
            for seg in lines_of_raster([(0, [last], ZERO), (v, pts, fl[4] if v == 4 else ZERO)]):
                if seg[0] != "move":
                    out.append((1, seg[1]))
            # lines_of_raster closes the contour at its end; drop that closing line
            if not (pts[-1][0] == last[0] and pts[-1][1] == last[1]):
                out.pop()
            last = pts[-1]
    return out


def stroke_polyline(poly, width):
    """path.rs:150-274 restated: contours first, then both offset sides."""
    width = F(width)
    half = F(0.5) * width
    contours = []          # (points, closed)
    cur = []
    closed = False
    started = False
    for v, p in poly + [(None, None)]:
        if v == 5:
            closed = True
        if v in (None, 0, 5) and cur:
            contours.append((cur, closed))
        if v == 0:
            cur = [p]
        elif v == 1:
            cur = cur + [p]
        elif v == 5:
            cur = []
    out = []

    def side(pts, closed, reverse):
        seq = pts[::-1] if reverse else pts
        first = pts[0] if closed == reverse else pts[-1]
        res = []
        prev, pn = first, (ZERO, ZERO)
        for i in range(len(seq) + 1):
            nxt = seq[i] if i < len(seq) else first
            if i < len(seq) and nxt[0] == prev[0] and nxt[1] == prev[1]:
                continue
            tx, ty = nxt[0] - prev[0], nxt[1] - prev[1]
            nn = (-ty, tx)
            ln = np.sqrt(nn[0] * nn[0] + nn[1] * nn[1])
            nn = (ZERO, ZERO) if ln == ZERO else (nn[0] * (ONE / ln), nn[1] * (ONE / ln))
            off = ONE / (ONE + (pn[0] * nn[0] + pn[1] * nn[1]))
            if abs(off) > F(2.0):
                res.append((prev[0] + half * pn[0], prev[1] + half * pn[1]))
                res.append((prev[0] + half * nn[0], prev[1] + half * nn[1]))
            else:
                k = half * off
                res.append((prev[0] + k * (pn[0] + nn[0]), prev[1] + k * (pn[1] + nn[1])))
            prev, pn = nxt, nn
        return res

    for pts, cl in contours:
        fwd = side(pts, cl, False)
        out += [(0 if j == 0 else 1, q) for j, q in enumerate(fwd)]
        if cl:
            out.append((5, None))
        bwd = side(pts, cl, True)
        out += [(0 if (j == 0 and cl) else 1, q) for j, q in enumerate(bwd)]
        out.append((5, None))
    return out


def commands_of_batch(batch, raster):
    """Device-space command list of one raster of a Batch."""
    from ochre_gb300.batch import FLOATS_PER_VERB
    fpo = np.concatenate([[0], np.cumsum(FLOATS_PER_VERB[batch.verbs])]).astype(np.int64)
    roff = batch.raster_fill_off if batch.raster_fill_off is not None else np.arange(batch.n_fills + 1)
    out = []
    for f in range(int(roff[raster]), int(roff[raster + 1])):
        xf = [F(v) for v in batch.fill_xf[f]]
        raw = batch.fill_flags is not None and bool(batch.fill_flags[f] & 1)
        if batch.fill_flags is not None and batch.fill_flags[f] & 2:
            c0, c1 = int(batch.fill_cmd_off[f]), int(batch.fill_cmd_off[f + 1])
            poly = path_polyline(batch.verbs[c0:c1], batch.pts[fpo[c0]:fpo[c1]])
            for v, q in stroke_polyline(poly, batch.fill_width[f]):
                pts = [] if q is None else [q if raw else apply(xf, q)]
                out.append((v, pts, ZERO))
            continue
        for c in range(int(batch.fill_cmd_off[f]), int(batch.fill_cmd_off[f + 1])):
            v = int(batch.verbs[c])
            fl = [F(q) for q in batch.pts[fpo[c]:fpo[c + 1]]]
            npts = {0: 1, 1: 1, 2: 2, 3: 3, 4: 2, 5: 0}[v]
            pts = [(fl[2 * k], fl[2 * k + 1]) for k in range(npts)]
            if not raw:
                pts = [apply(xf, q) for q in pts]
            out.append((v, pts, fl[4] if v == 4 else ZERO))
    return out
