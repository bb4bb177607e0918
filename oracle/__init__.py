"""ORACLE — test infrastructure only.

ctypes wrapper over ``ochre_oracle.c``, a strict-f32 CPU restatement of ochre
0.2.0's rasterizer (``src/rasterizer.rs``, ``src/path.rs``, ``src/geom.rs``).
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use it, as the checker; the product never imports it.

Parity with the reference: UNPINNED.  The reference is a Rust crate that
cannot be built here (no rustc/cargo) and ships no tests or golden vectors.
The restatement is cross-checked against an independent numpy-float32
restatement (``tests/oracle_py.py``) and hand-derived known answers.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libochre_oracle.so")

CFLAGS = ["-O3", "-ffp-contract=off", "-fno-fast-math", "-fexcess-precision=standard",
          "-fno-strict-aliasing", "-std=c11", "-fPIC", "-shared", "-pthread"]


def build(force: bool = False) -> str:
    """Compile the oracle into oracle/_build/libochre_oracle.so."""
    src = os.path.join(_HERE, "ochre_oracle.c")
    hdr = os.path.join(_HERE, "ochre_oracle.h")
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return _LIB_PATH
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", *CFLAGS, "-o", tmp, src, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


class _Batch(ctypes.Structure):
    _fields_ = [
        ("verbs", ctypes.c_void_p), ("n_cmds", ctypes.c_uint64),
        ("pts", ctypes.c_void_p), ("n_floats", ctypes.c_uint64),
        ("fill_cmd_off", ctypes.c_void_p), ("fill_xf", ctypes.c_void_p),
        ("fill_flags", ctypes.c_void_p), ("n_fills", ctypes.c_uint32),
        ("raster_fill_off", ctypes.c_void_p), ("n_rasters", ctypes.c_uint32),
        ("fill_width", ctypes.c_void_p),
    ]


class _Result(ctypes.Structure):
    _fields_ = [
        ("n_rasters", ctypes.c_uint32),
        ("n_tiles", ctypes.c_uint64), ("n_spans", ctypes.c_uint64), ("n_lines", ctypes.c_uint64),
        ("tile_xy", ctypes.c_void_p), ("tile_alpha", ctypes.c_void_p), ("tile_cov", ctypes.c_void_p),
        ("span_xy", ctypes.c_void_p), ("span_w", ctypes.c_void_p), ("span_tile", ctypes.c_void_p),
        ("raster_tile_off", ctypes.c_void_p), ("raster_span_off", ctypes.c_void_p),
        ("raster_line_off", ctypes.c_void_p), ("raster_stats", ctypes.c_void_p),
        ("lines", ctypes.c_void_p), ("line_ninc", ctypes.c_void_p),
        ("error_raster", ctypes.c_uint32),
    ]


_lib = None


def _load():
    global _lib
    if _lib is None:
        path = build()
        lib = ctypes.CDLL(path)
        lib.ochre_oracle_run.argtypes = [ctypes.POINTER(_Batch), ctypes.c_int, ctypes.c_int,
                                         ctypes.POINTER(ctypes.POINTER(_Result))]
        lib.ochre_oracle_run.restype = ctypes.c_int
        lib.ochre_oracle_free.argtypes = [ctypes.POINTER(_Result)]
        lib.ochre_oracle_free.restype = None
        lib.ochre_oracle_cov64.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p,
                                           ctypes.c_void_p]
        lib.ochre_oracle_cov64.restype = ctypes.c_int
        lib.ochre_oracle_seg_counts.argtypes = [ctypes.POINTER(_Batch), ctypes.c_void_p]
        lib.ochre_oracle_seg_counts.restype = ctypes.c_int
        lib.ochre_oracle_diff64.argtypes = [ctypes.POINTER(_Batch), ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_void_p,
                                            ctypes.c_void_p]
        lib.ochre_oracle_diff64.restype = ctypes.c_int
        lib.ochre_oracle_backward64.argtypes = [ctypes.POINTER(_Batch), ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.ochre_oracle_backward64.restype = ctypes.c_int
        lib.ochre_oracle_forward64.argtypes = [ctypes.POINTER(_Batch), ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                               ctypes.c_void_p]
        lib.ochre_oracle_forward64.restype = ctypes.c_int
        lib.ochre_oracle_stroke.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_float,
                                            ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_uint64),
                                            ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_uint64)]
        lib.ochre_oracle_stroke.restype = ctypes.c_int
        lib.ochre_oracle_composite.argtypes = [ctypes.c_uint32] + [ctypes.c_void_p] * 7 + [ctypes.c_uint32,
                                                                                           ctypes.c_uint32,
                                                                                           ctypes.c_void_p]
        lib.ochre_oracle_composite.restype = None
        lib.free.argtypes = [ctypes.c_void_p]
        lib.free.restype = None
        _lib = lib
    return _lib


def _copy(ptr, dtype, count):
    if count == 0 or not ptr:
        return np.zeros(0, dtype=dtype)
    buf = (ctypes.c_char * (count * np.dtype(dtype).itemsize)).from_address(ptr)
    return np.frombuffer(buf, dtype=dtype).copy()


def _as_batch(batch):
    keep = []

    def p(a, dtype):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dtype)
        keep.append(a)
        return a.ctypes.data

    b = _Batch()
    b.verbs = p(batch.verbs, np.uint8)
    b.n_cmds = len(batch.verbs)
    b.pts = p(batch.pts, np.float32)
    b.n_floats = len(batch.pts)
    b.fill_cmd_off = p(batch.fill_cmd_off, np.uint32)
    b.fill_xf = p(batch.fill_xf, np.float32)
    b.fill_flags = p(batch.fill_flags, np.uint8)
    b.n_fills = len(batch.fill_cmd_off) - 1
    b.raster_fill_off = p(batch.raster_fill_off, np.uint32)
    b.n_rasters = batch.n_rasters
    b.fill_width = p(getattr(batch, "fill_width", None), np.float32)
    return b, keep


def run(batch, threads: int = 1, want_cov: bool = False, capture_lines: bool = False,
        signed_cov: bool = False) -> dict:
    """Rasterize every raster of ``batch`` on the CPU.

    ``batch`` has the attributes of ``ochre_gb300.batch.Batch`` (numpy arrays
    in the C-ABI layout).  Returns a dict of numpy arrays in the same layout as
    the GPU result plus per-raster statistics.
    """
    lib = _load()
    b, keep = _as_batch(batch)
    flags = (1 if want_cov else 0) | (2 if capture_lines else 0) | (4 if signed_cov else 0)
    res_p = ctypes.POINTER(_Result)()
    st = lib.ochre_oracle_run(ctypes.byref(b), int(threads), flags, ctypes.byref(res_p))
    if not res_p:
        raise RuntimeError(f"oracle failed with status {st}")
    try:
        r = res_p.contents
        nr, nt, ns, nl = r.n_rasters, r.n_tiles, r.n_spans, r.n_lines
        out = {
            "status": st,
            "tile_xy": _copy(r.tile_xy, np.int16, 2 * nt).reshape(nt, 2),
            "tile_alpha": _copy(r.tile_alpha, np.uint8, 64 * nt).reshape(nt, 64),
            "span_xy": _copy(r.span_xy, np.int16, 2 * ns).reshape(ns, 2),
            "span_w": _copy(r.span_w, np.uint16, ns),
            "span_tile": _copy(r.span_tile, np.uint32, ns),
            "raster_tile_off": _copy(r.raster_tile_off, np.uint64, nr + 1),
            "raster_span_off": _copy(r.raster_span_off, np.uint64, nr + 1),
            "raster_stats": _copy(r.raster_stats, np.uint64, 3 * nr).reshape(nr, 3),
        }
        if want_cov:
            out["tile_cov"] = _copy(r.tile_cov, np.float32, 64 * nt).reshape(nt, 64)
        if capture_lines:
            out["lines"] = _copy(r.lines, np.float32, 4 * nl).reshape(nl, 4)
            out["line_ninc"] = _copy(r.line_ninc, np.uint32, nl)
            out["raster_line_off"] = _copy(r.raster_line_off, np.uint64, nr + 1)
        return out
    finally:
        lib.ochre_oracle_free(res_p)


def cov64(lines: np.ndarray, raster_line_off: np.ndarray, rects: np.ndarray) -> list:
    """FP64 analytic coverage |sum| of f32 lines (from run(capture_lines=True))
    over one pixel rectangle (x0, y0, w, h) per raster; returns one [h, w]
    float64 image per raster."""
    lib = _load()
    lines = np.ascontiguousarray(lines, dtype=np.float32)
    off = np.ascontiguousarray(raster_line_off, dtype=np.uint64)
    rects = np.ascontiguousarray(rects, dtype=np.int32).reshape(-1, 4)
    n = len(rects)
    total = int((rects[:, 2].astype(np.int64) * rects[:, 3]).sum())
    out = np.zeros(max(total, 1), dtype=np.float64)
    st = lib.ochre_oracle_cov64(lines.ctypes.data, off.ctypes.data, n, rects.ctypes.data, out.ctypes.data)
    if st:
        raise RuntimeError(f"oracle cov64 failed with status {st}")
    imgs, b = [], 0
    for x0, y0, w, h in rects:
        imgs.append(out[b:b + w * h].reshape(h, w))
        b += w * h
    return imgs


def tile_cov_error_vs_fp64(batch, gpu_tile_xy, gpu_tile_cov, gpu_raster_tile_off) -> dict:
    """Pre-quantisation coverage error of a result (per-tile |accum + area|,
    64 per tile) against the FP64 analytic coverage of the same f32 lines, at
    every tile pixel.  Returns max / mean absolute error."""
    ref = run(batch, capture_lines=True)
    R = batch.n_rasters
    rects = np.zeros((R, 4), np.int32)
    for r in range(R):
        t0, t1 = int(gpu_raster_tile_off[r]), int(gpu_raster_tile_off[r + 1])
        xy = gpu_tile_xy[t0:t1].astype(np.int64)
        rects[r] = (xy[:, 0].min(), xy[:, 1].min(), xy[:, 0].max() - xy[:, 0].min() + 8,
                    xy[:, 1].max() - xy[:, 1].min() + 8)
    imgs = cov64(ref["lines"], ref["raster_line_off"], rects)
    errs = []
    for r in range(R):
        t0, t1 = int(gpu_raster_tile_off[r]), int(gpu_raster_tile_off[r + 1])
        x0, y0 = rects[r, 0], rects[r, 1]
        img = imgs[r]
        for t in range(t0, t1):
            tx, ty = int(gpu_tile_xy[t, 0]) - x0, int(gpu_tile_xy[t, 1]) - y0
            block = img[ty:ty + 8, tx:tx + 8].reshape(64)
            errs.append(np.abs(gpu_tile_cov[t].astype(np.float64) - block))
    e = np.concatenate(errs) if errs else np.zeros(1)
    return {"max_abs": float(e.max()), "mean_abs": float(e.mean()), "pixels": int(e.size)}


def stroke(verbs, pts, width: float):
    """Rasterizer::stroke's preprocessing of one path (path.rs:113-274):
    returns (verbs, pts) of the Move / Line / Close path that is filled."""
    lib = _load()
    v = np.ascontiguousarray(verbs, np.uint8)
    p = np.ascontiguousarray(pts, np.float32)
    ov, op = ctypes.c_void_p(), ctypes.c_void_p()
    n, nf = ctypes.c_uint64(), ctypes.c_uint64()
    st = lib.ochre_oracle_stroke(v.ctypes.data if len(v) else None, len(v), p.ctypes.data if len(p) else None,
                                 float(width), ctypes.byref(ov), ctypes.byref(n), ctypes.byref(op), ctypes.byref(nf))
    if st:
        raise RuntimeError(f"oracle stroke failed with status {st}")
    try:
        out_v = _copy(ov.value, np.uint8, n.value)
        out_p = _copy(op.value, np.float32, nf.value)
    finally:
        lib.free(ov)
        lib.free(op)
    return out_v, out_p


def composite(result: dict, n_rasters: int, colors, w: int, h: int, canvas=None) -> np.ndarray:
    """Headless compositing of a result (dict of run()'s layout) with one
    RGBA8 colour per raster onto an RGBA8 [h, w, 4] canvas (white if None)."""
    lib = _load()
    cv = np.full((h, w, 4), 255, np.uint8) if canvas is None else np.ascontiguousarray(canvas, np.uint8).copy()
    arr = lambda k, dt: np.ascontiguousarray(result[k], dt)
    keep = [arr("tile_xy", np.int16), arr("tile_alpha", np.uint8), arr("raster_tile_off", np.uint64),
            arr("span_xy", np.int16), arr("span_w", np.uint16), arr("raster_span_off", np.uint64),
            np.ascontiguousarray(colors, np.uint8).reshape(-1)]
    ptr = lambda a: a.ctypes.data if a.size else None
    lib.ochre_oracle_composite(n_rasters, *[ptr(a) for a in keep], w, h, cv.ctypes.data)
    return cv


def seg_counts(batch) -> np.ndarray:
    """Lines the f32 flattening gives each command (0 for non-curves)."""
    lib = _load()
    b, keep = _as_batch(batch)
    out = np.zeros(max(len(batch.verbs), 1), np.uint32)
    st = lib.ochre_oracle_seg_counts(ctypes.byref(b), out.ctypes.data)
    if st:
        raise RuntimeError(f"oracle seg_counts failed with status {st}")
    return out[:len(batch.verbs)]


def diff64(batch, w: int, h: int, target: np.ndarray, counts=None, grad: bool = True):
    """FP64 differentiable model: returns (loss, dL/dpts, dL/dxf) for a
    ``w`` x ``h`` canvas per raster against ``target`` ([R, h, w]); line
    counts of curves are held at ``counts`` (default: the f32 flattening's)."""
    lib = _load()
    b, keep = _as_batch(batch)
    counts = seg_counts(batch) if counts is None else np.ascontiguousarray(counts, np.uint32)
    target = np.ascontiguousarray(target, np.float64)
    assert target.size == batch.n_rasters * w * h
    loss = ctypes.c_double()
    dpts = np.zeros(max(len(batch.pts), 1), np.float64)
    dxf = np.zeros(max(6 * (len(batch.fill_cmd_off) - 1), 1), np.float64)
    st = lib.ochre_oracle_diff64(ctypes.byref(b), counts.ctypes.data if counts.size else None, int(w), int(h),
                                 target.ctypes.data, ctypes.byref(loss),
                                 dpts.ctypes.data if grad else None, dxf.ctypes.data if grad else None)
    if st:
        raise RuntimeError(f"oracle diff64 failed with status {st}")
    return loss.value, dpts[:len(batch.pts)], dxf[:6 * (len(batch.fill_cmd_off) - 1)].reshape(-1, 6)


def backward64(batch, w: int, h: int, dl_ds: np.ndarray, counts=None):
    """FP64 backward of the same model from a given dL/dS image ([R, h, w]);
    returns (dL/dpts, dL/dxf)."""
    lib = _load()
    b, keep = _as_batch(batch)
    counts = seg_counts(batch) if counts is None else np.ascontiguousarray(counts, np.uint32)
    g = np.ascontiguousarray(dl_ds, np.float64)
    assert g.size == batch.n_rasters * w * h
    dpts = np.zeros(max(len(batch.pts), 1), np.float64)
    dxf = np.zeros(max(6 * (len(batch.fill_cmd_off) - 1), 1), np.float64)
    st = lib.ochre_oracle_backward64(ctypes.byref(b), counts.ctypes.data if counts.size else None, int(w), int(h),
                                     g.ctypes.data, dpts.ctypes.data, dxf.ctypes.data)
    if st:
        raise RuntimeError(f"oracle backward64 failed with status {st}")
    return dpts[:len(batch.pts)], dxf[:6 * (len(batch.fill_cmd_off) - 1)].reshape(-1, 6)


def forward64(batch, w: int, h: int, counts=None) -> np.ndarray:
    """The FP64 model's signed pre-quantisation sums S = accum + area of every
    pixel, [R, h, w] (the all-double forward of diff64)."""
    lib = _load()
    b, keep = _as_batch(batch)
    counts = seg_counts(batch) if counts is None else np.ascontiguousarray(counts, np.uint32)
    out = np.zeros(max(batch.n_rasters * w * h, 1), np.float64)
    st = lib.ochre_oracle_forward64(ctypes.byref(b), counts.ctypes.data if counts.size else None, int(w), int(h),
                                    out.ctypes.data)
    if st:
        raise RuntimeError(f"oracle forward64 failed with status {st}")
    return out[:batch.n_rasters * w * h].reshape(batch.n_rasters, h, w)


def _tile_images(batch, w: int, h: int):
    """Signed pre-quantisation sums at boundary-tile pixels (f32 restatement),
    the boundary-tile mask and the span mask, each [R, h, w] on a canvas at
    the origin."""
    ref = run(batch, want_cov=True, signed_cov=True)
    R = batch.n_rasters
    S = np.zeros((R, h + 8, w + 8), np.float32)
    T = np.zeros((R, h + 8, w + 8), bool)
    P = np.zeros((R, h + 8, w + 8), bool)
    for r in range(R):
        t0, t1 = int(ref["raster_tile_off"][r]), int(ref["raster_tile_off"][r + 1])
        for t in range(t0, t1):
            x, y = int(ref["tile_xy"][t, 0]), int(ref["tile_xy"][t, 1])
            if x <= -8 or y <= -8 or x >= w or y >= h:
                continue
            blk = ref["tile_cov"][t].reshape(8, 8)
            xs, ys = max(x, 0), max(y, 0)
            S[r, ys:y + 8, xs:x + 8] = blk[ys - y:, xs - x:]
            T[r, ys:y + 8, xs:x + 8] = True
        s0, s1 = int(ref["raster_span_off"][r]), int(ref["raster_span_off"][r + 1])
        for s in range(s0, s1):
            x, y, sw = int(ref["span_xy"][s, 0]), int(ref["span_xy"][s, 1]), int(ref["span_w"][s])
            if y <= -8 or y >= h or x + sw <= 0 or x >= w:
                continue
            P[r, max(y, 0):y + 8, max(x, 0):min(x + sw, w)] = True
    return S[:, :h, :w], T[:, :h, :w], P[:, :h, :w]


def coverage_image(batch, w: int, h: int) -> np.ndarray:
    """f32 model coverage min(|accum + area|, 1) of each raster on a w x h
    canvas at the origin, from the f32 restatement (tiles) and its spans."""
    S, T, P = _tile_images(batch, w, h)
    return np.where(T, np.minimum(np.abs(S), 1.0), np.where(P, 1.0, 0.0)).astype(np.float32)


def adjoint64(batch, w: int, h: int, target: np.ndarray, counts=None):
    """The FP64 reference gradient of the f32 model: the loss and dL/dS of
    the f32 forward (the reference's arithmetic, as the GPU computes it),
    then the adjoint through the lines, the flattening and the transforms in
    double precision.  Returns (loss, dL/dpts, dL/dxf)."""
    S, T, P = _tile_images(batch, w, h)
    c = np.where(T, np.minimum(np.abs(S), 1.0), np.where(P, 1.0, 0.0)).astype(np.float64)
    d = c - np.asarray(target, np.float64).reshape(c.shape)
    g = np.where(T & (np.abs(S) < 1.0), np.sign(S) * 2.0 * d, 0.0)
    dp, dx = backward64(batch, w, h, g, counts)
    return float((d * d).sum()), dp, dx


if __name__ == "__main__":  # pragma: no cover
    print(build(force="--force" in sys.argv))
