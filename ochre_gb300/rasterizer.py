"""Python mirror of ochre's public API over the C ABI.

``Vec2``, ``Mat2x2``, ``Transform`` (src/geom.rs), ``PathCmd`` (src/path.rs:5-12),
``TileBuilder`` and ``Rasterizer`` (src/rasterizer.rs:12-268) keep the
reference's names, argument meaning and call order; rasterization runs on the
GPU through libochre_gpu.so.  ``GpuContext`` exposes the batched entry points
(many independent rasterizers per call) used by the benchmark.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np

from . import _lib
from .batch import (CLOSE, CONIC, CUBIC, FLOATS_PER_VERB, IDENTITY, LINE, MOVE, QUADRATIC, Batch,
                    BatchBuilder)

TILE_SIZE = 8  # src/rasterizer.rs:4


# ---------------------------------------------------------------------------
# geom.rs
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class Vec2:
    x: float
    y: float


@dataclass(frozen=True)
class Mat2x2:
    """Row-major 2x2 matrix (geom.rs:133)."""
    m: tuple

    @staticmethod
    def new(a: float, b: float, c: float, d: float) -> "Mat2x2":
        return Mat2x2((a, b, c, d))

    @staticmethod
    def id() -> "Mat2x2":
        return Mat2x2((1.0, 0.0, 0.0, 1.0))

    @staticmethod
    def scale(s: float) -> "Mat2x2":
        return Mat2x2((s, 0.0, 0.0, s))

    @staticmethod
    def rotate(angle: float) -> "Mat2x2":
        """geom.rs:152-154: [cos, sin, -sin, cos] (evaluated in f32)."""
        a = np.float32(angle)
        c, s = float(np.cos(a)), float(np.sin(a))
        return Mat2x2((c, s, -s, c))


@dataclass(frozen=True)
class Transform:
    matrix: Mat2x2
    offset: Vec2

    @staticmethod
    def new(matrix: Mat2x2, offset: Vec2) -> "Transform":
        return Transform(matrix, offset)

    @staticmethod
    def id() -> "Transform":
        return Transform(Mat2x2.id(), Vec2(0.0, 0.0))

    @staticmethod
    def translate(x: float, y: float) -> "Transform":
        return Transform(Mat2x2.id(), Vec2(x, y))

    @staticmethod
    def scale(s: float) -> "Transform":
        return Transform(Mat2x2.scale(s), Vec2(0.0, 0.0))

    @staticmethod
    def rotate(angle: float) -> "Transform":
        return Transform(Mat2x2.rotate(angle), Vec2(0.0, 0.0))

    def then(self, t: "Transform") -> "Transform":
        """geom.rs:252-257, in f32."""
        f = np.float32
        a, b = [f(v) for v in t.matrix.m], [f(v) for v in self.matrix.m]
        m = (a[0] * b[0] + a[1] * b[2], a[0] * b[1] + a[1] * b[3], a[2] * b[0] + a[3] * b[2], a[2] * b[1] + a[3] * b[3])
        ox, oy = f(self.offset.x), f(self.offset.y)
        o = (a[0] * ox + a[1] * oy + f(t.offset.x), a[2] * ox + a[3] * oy + f(t.offset.y))
        return Transform(Mat2x2(tuple(float(v) for v in m)), Vec2(float(o[0]), float(o[1])))

    def as_array(self) -> np.ndarray:
        return np.array([*self.matrix.m, self.offset.x, self.offset.y], dtype=np.float32)


# ---------------------------------------------------------------------------
# path.rs
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class PathCmd:
    """One path command: use the constructors Move/Line/Quadratic/Cubic/Conic/Close."""
    verb: int
    floats: tuple = ()

    @staticmethod
    def Move(p: Vec2) -> "PathCmd":
        return PathCmd(MOVE, (p.x, p.y))

    @staticmethod
    def Line(p: Vec2) -> "PathCmd":
        return PathCmd(LINE, (p.x, p.y))

    @staticmethod
    def Quadratic(c: Vec2, p: Vec2) -> "PathCmd":
        return PathCmd(QUADRATIC, (c.x, c.y, p.x, p.y))

    @staticmethod
    def Cubic(c1: Vec2, c2: Vec2, p: Vec2) -> "PathCmd":
        return PathCmd(CUBIC, (c1.x, c1.y, c2.x, c2.y, p.x, p.y))

    @staticmethod
    def Conic(c: Vec2, p: Vec2, w: float) -> "PathCmd":
        return PathCmd(CONIC, (c.x, c.y, p.x, p.y, w))

    @staticmethod
    def Close() -> "PathCmd":
        return PathCmd(CLOSE, ())


def encode_path(path: Sequence[PathCmd]) -> tuple[np.ndarray, np.ndarray]:
    verbs = np.array([c.verb for c in path], dtype=np.uint8)
    pts = np.array([v for c in path for v in c.floats], dtype=np.float32)
    return verbs, pts


# ---------------------------------------------------------------------------
# rasterizer.rs
# ---------------------------------------------------------------------------
class TileBuilder:
    """rasterizer.rs:12-22.  Subclass and override tile() and span()."""

    def tile(self, x: int, y: int, data: bytes) -> None:  # pragma: no cover - interface
        raise NotImplementedError

    def span(self, x: int, y: int, width: int) -> None:  # pragma: no cover - interface
        raise NotImplementedError


_default_ctx: Optional["GpuContext"] = None


def default_context() -> "GpuContext":
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = GpuContext(0)
    return _default_ctx


class Rasterizer:
    """rasterizer.rs:40-268: Rasterizer::new / move_to / line_to / command /
    fill / finish.  Commands are buffered on the host; finish() rasterizes on
    the GPU and calls the builder in the reference's order."""

    def __init__(self, ctx: Optional["GpuContext"] = None):
        self._ctx = ctx or default_context()
        L = _lib.load()
        h = ctypes.c_void_p()
        _lib.check(L.ochre_rasterizer_new(self._ctx.handle, ctypes.byref(h)), "Rasterizer::new")
        self._h = h

    @staticmethod
    def new(ctx: Optional["GpuContext"] = None) -> "Rasterizer":
        return Rasterizer(ctx)

    def _live(self):
        if self._h is None:
            raise RuntimeError("Rasterizer used after finish()")
        return self._h

    def move_to(self, point: Vec2) -> None:
        _lib.check(_lib.load().ochre_rasterizer_move_to(self._live(), point.x, point.y), "move_to")

    def line_to(self, point: Vec2) -> None:
        _lib.check(_lib.load().ochre_rasterizer_line_to(self._live(), point.x, point.y), "line_to")

    def command(self, cmd: PathCmd) -> None:
        f = (ctypes.c_float * max(1, len(cmd.floats)))(*cmd.floats)
        _lib.check(_lib.load().ochre_rasterizer_command(self._live(), cmd.verb, f), "command")

    def fill(self, path: Sequence[PathCmd], transform: Transform) -> None:
        verbs, pts = encode_path(path)
        xf = transform.as_array()
        _lib.check(_lib.load().ochre_rasterizer_fill(
            self._live(), verbs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), len(verbs),
            pts.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(pts),
            xf.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "fill")

    def stroke(self, path: Sequence[PathCmd], width: float, transform: Transform) -> None:
        """rasterizer.rs:169-171: the path stroked with ``width`` (in its own
        space), then filled with ``transform``."""
        verbs, pts = encode_path(path)
        xf = transform.as_array()
        _lib.check(_lib.load().ochre_rasterizer_stroke(
            self._live(), verbs.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), len(verbs),
            pts.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), len(pts), float(width),
            xf.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "stroke")

    def finish(self, builder: TileBuilder) -> None:
        h = self._live()
        self._h = None  # finish consumes the rasterizer
        errors = []

        def on_tile(_user, x, y, data):
            try:
                builder.tile(int(x), int(y), ctypes.string_at(data, 64))
            except BaseException as e:  # pragma: no cover - surfaced below
                errors.append(e)

        def on_span(_user, x, y, w):
            try:
                builder.span(int(x), int(y), int(w))
            except BaseException as e:  # pragma: no cover
                errors.append(e)

        st = _lib.load().ochre_rasterizer_finish(h, _lib.TILE_FN(on_tile), _lib.SPAN_FN(on_span), None)
        if errors:
            raise errors[0]
        _lib.check(st, "finish")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _lib._lib is not None:
            _lib._lib.ochre_rasterizer_free(h)
            self._h = None


# ---------------------------------------------------------------------------
# Batched entry points
# ---------------------------------------------------------------------------
CUDA_STREAM_LEGACY = 1   # cudaStreamLegacy: the legacy default stream


def stream_arg(stream: Optional[int]) -> Optional[int]:
    """A cudaStream_t for the C ABI.  None: the context's own stream (NULL).
    A stream handle of 0 (torch's default stream is the legacy default
    stream) becomes cudaStreamLegacy, so that the work is ordered with what
    torch runs there; NULL would mean the context's own (non-blocking)
    stream instead."""
    if stream is None:
        return None
    return int(stream) if int(stream) != 0 else CUDA_STREAM_LEGACY


class Graph:
    """A captured fill -> finish launch chain for one DeviceBatch (its device
    pointers and counts fixed; the values behind them may change between
    launches).  Owns its buffers; results are device pointers valid until the
    next launch."""

    def __init__(self, ctx: "GpuContext", dbatch: "DeviceBatch", headroom: float = 1.25, _create=None):
        L = _lib.load()
        h = ctypes.c_void_p()
        self.dbatch = dbatch   # keeps the device storage alive
        self.n_rasters = dbatch.batch.n_rasters
        self._ctx = ctx
        if _create is None:
            _lib.check(L.ochre_graph_create(ctx.handle, ctypes.byref(dbatch.c), ctypes.c_float(headroom),
                                            ctypes.byref(h)), "ochre_graph_create")
        else:
            _create(h)
        self.handle = h

    def launch(self, stream: Optional[int] = None) -> _lib.Result:
        r = _lib.Result()
        _lib.check(_lib.load().ochre_graph_launch(self.handle, ctypes.byref(r), stream_arg(stream)),
                   "ochre_graph_launch")
        return r

    def rasterize(self, stream: Optional[int] = None) -> dict:
        """launch() with the result copied to numpy arrays."""
        return self._ctx.device_result_to_numpy(self.launch(stream), self.n_rasters)

    def stats(self) -> _lib.Stats:
        st = _lib.Stats()
        _lib.check(_lib.load().ochre_graph_last_stats(self.handle, ctypes.byref(st)))
        return st

    def info(self) -> dict:
        k, r, f = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        _lib.check(_lib.load().ochre_graph_info(self.handle, ctypes.byref(k), ctypes.byref(r), ctypes.byref(f)))
        return {"kernels": k.value, "replans": r.value, "fused": bool(f.value)}

    def close(self) -> None:
        if getattr(self, "handle", None) is not None:
            _lib.load().ochre_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

def _c_batch(verbs_p, n_cmds, pts_p, n_floats, off_p, xf_p, flags_p, n_fills, roff_p, n_rasters,
             width_p=None) -> _lib.Batch:
    b = _lib.Batch()
    b.verbs, b.n_cmds, b.pts, b.n_floats = verbs_p, n_cmds, pts_p, n_floats
    b.fill_cmd_off, b.fill_xf, b.fill_flags, b.n_fills = off_p, xf_p, flags_p, n_fills
    b.raster_fill_off, b.n_rasters = roff_p, n_rasters
    b.fill_width = width_p
    return b


def _host_c_batch(batch: Batch):
    """(the C struct over the batch's host arrays, the arrays it points into)."""
    keep = []

    def p(a, dt):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return a.ctypes.data

    c = _c_batch(p(batch.verbs, np.uint8), batch.n_cmds, p(batch.pts, np.float32), len(batch.pts),
                 p(batch.fill_cmd_off, np.uint32), p(batch.fill_xf, np.float32), p(batch.fill_flags, np.uint8),
                 batch.n_fills, p(batch.raster_fill_off, np.uint32), batch.n_rasters,
                 p(getattr(batch, "fill_width", None), np.float32))
    return c, keep


def validate_batch(batch: Batch) -> None:
    """ochre_validate_batch: the structural check ochre_gpu_rasterize makes
    before its first copy (no GPU needed); raises OchreError."""
    c, keep = _host_c_batch(batch)
    _lib.check(_lib.load().ochre_validate_batch(ctypes.byref(c)), "validate_batch")


class DeviceBatch:
    """A Batch resident in device memory (torch CUDA tensors as storage)."""

    def __init__(self, batch: Batch, device: int = 0):
        import torch
        dev = torch.device("cuda", device)
        self.batch = batch
        t = lambda a, dt: torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(dev)
        self.verbs = t(batch.verbs if len(batch.verbs) else np.zeros(1, np.uint8), np.uint8)
        self.pts = t(batch.pts if len(batch.pts) else np.zeros(1, np.float32), np.float32)
        self.fill_off = t(batch.fill_cmd_off.astype(np.int32), np.int32)
        self.fill_xf = t(batch.fill_xf.reshape(-1) if batch.n_fills else np.zeros(6, np.float32), np.float32)
        self.fill_flags = t(batch.fill_flags, np.uint8) if batch.fill_flags is not None else None
        self.raster_off = (t(batch.raster_fill_off.astype(np.int32), np.int32)
                           if batch.raster_fill_off is not None else None)
        fw = getattr(batch, "fill_width", None)
        self.fill_width = t(fw, np.float32) if fw is not None and batch.n_fills else None
        self.c = _c_batch(self.verbs.data_ptr(), batch.n_cmds, self.pts.data_ptr(), len(batch.pts),
                          self.fill_off.data_ptr(), self.fill_xf.data_ptr(),
                          self.fill_flags.data_ptr() if self.fill_flags is not None else None,
                          batch.n_fills, self.raster_off.data_ptr() if self.raster_off is not None else None,
                          batch.n_rasters, self.fill_width.data_ptr() if self.fill_width is not None else None)

    def input_bytes(self) -> int:
        return self.batch.input_bytes()


class DiffGraph(Graph):
    """A captured differentiable step on fixed buffers: ``cov`` [n_rasters, h,
    w], ``dl_dcov`` (same shape), ``loss`` [1] float64, ``dl_dpts``
    [n_floats] and ``dl_dxf`` [n_fills, 6] (CUDA tensors), rewritten by every
    launch.  The values behind the batch and ``target`` may change between
    launches."""

    def __init__(self, ctx: "GpuContext", dbatch: "DeviceBatch", w: int, h: int, target, headroom: float = 1.25):
        import torch
        b = dbatch.batch
        dev = target.device
        self.target = target
        self.cov = torch.empty((b.n_rasters, h, w), dtype=torch.float32, device=dev)
        self.dl_dcov = torch.empty_like(self.cov)
        self.loss = torch.empty(1, dtype=torch.float64, device=dev)
        self.dl_dpts = torch.empty(max(1, len(b.pts)), dtype=torch.float32, device=dev)
        self.dl_dxf = torch.empty((max(1, b.n_fills), 6), dtype=torch.float32, device=dev)

        def create(hnd):
            _lib.check(_lib.load().ochre_graph_create_diff(
                ctx.handle, ctypes.byref(dbatch.c), w, h, target.data_ptr(), self.cov.data_ptr(),
                self.dl_dcov.data_ptr(), self.loss.data_ptr(), self.dl_dpts.data_ptr(), self.dl_dxf.data_ptr(),
                ctypes.c_float(headroom), ctypes.byref(hnd)), "ochre_graph_create_diff")
        super().__init__(ctx, dbatch, headroom, _create=create)


def _np_from(ptr, dtype, count):
    if count == 0 or not ptr:
        return np.zeros(0, dtype=dtype)
    buf = (ctypes.c_char * (count * np.dtype(dtype).itemsize)).from_address(ptr)
    return np.frombuffer(buf, dtype=dtype).copy()


class GpuContext:
    """One libochre_gpu context (device + stream + buffers)."""

    def __init__(self, device: int = 0, want_cov: bool = False, profile: bool = False, chain_only: bool = False):
        L = _lib.load()
        h = ctypes.c_void_p()
        self.want_cov = want_cov
        self.profile = profile
        self.chain_only = chain_only
        _lib.check(L.ochre_gpu_create(ctypes.byref(h), int(device), self._flags()), "ochre_gpu_create")
        self.handle = h
        self.device = device
        # launch shapes chosen earlier by the autotuner on this GPU, if any
        try:
            from . import autotune
            params = autotune.cached(device)
        except Exception:
            params = None
        if params:
            autotune.apply(self, params)

    def _flags(self) -> int:
        return ((_lib.CTX_WANT_COV if self.want_cov else 0) | (_lib.CTX_PROFILE if self.profile else 0)
                | (_lib.CTX_CHAIN_ONLY if self.chain_only else 0))

    def set_chain_only(self, on: bool) -> None:
        self.chain_only = on
        _lib.check(_lib.load().ochre_gpu_set_flags(self.handle, self._flags()))

    def set_want_cov(self, on: bool) -> None:
        self.want_cov = on
        _lib.check(_lib.load().ochre_gpu_set_flags(self.handle, self._flags()))

    def set_profile(self, on: bool) -> None:
        self.profile = on
        _lib.check(_lib.load().ochre_gpu_set_flags(self.handle, self._flags()))

    def timings(self) -> list:
        """[(kernel name, ms)] of the last run (needs profile=True)."""
        n = ctypes.c_uint32()
        L = _lib.load()
        _lib.check(L.ochre_gpu_last_timings(self.handle, None, 0, ctypes.byref(n)))
        arr = (_lib.KernelTime * max(1, n.value))()
        _lib.check(L.ochre_gpu_last_timings(self.handle, arr, n.value, ctypes.byref(n)))
        return [(arr[i].name.decode(), float(arr[i].ms)) for i in range(n.value)]

    def close(self) -> None:
        if self.handle is not None:
            _lib.load().ochre_gpu_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def rasterize(self, batch: Batch) -> dict:
        """Host buffers in, host arrays out (copies the batch to the device,
        rasterizes, copies results back)."""
        r = self.rasterize_raw(batch)
        return self._result_to_numpy(r, batch.n_rasters)

    def rasterize_raw(self, batch: Batch) -> _lib.Result:
        """ochre_gpu_rasterize itself: results stay in the context's pinned
        host buffers (valid until the next call)."""
        c, keep = _host_c_batch(batch)
        r = _lib.Result()
        _lib.check(_lib.load().ochre_gpu_rasterize(self.handle, ctypes.byref(c), ctypes.byref(r)), "rasterize")
        return r

    def rasterize_device(self, dbatch: DeviceBatch, stream: Optional[int] = None) -> _lib.Result:
        """Device buffers in, device result (pointers owned by the context)."""
        r = _lib.Result()
        _lib.check(_lib.load().ochre_gpu_rasterize_device(self.handle, ctypes.byref(dbatch.c), ctypes.byref(r),
                                                          stream_arg(stream)), "rasterize_device")
        return r

    def graph(self, dbatch: DeviceBatch, headroom: float = 1.25) -> "Graph":
        """The launch chain of rasterize_device for this batch, captured into a
        CUDA graph (ochre_graph_create)."""
        return Graph(self, dbatch, headroom)

    def graph_diff(self, dbatch: DeviceBatch, w: int, h: int, target, headroom: float = 1.25) -> "DiffGraph":
        """One differentiable step (render_coverage, l2_loss against ``target``
        [n_rasters, h, w], fill_backward) captured into a CUDA graph
        (ochre_graph_create_diff); its output tensors are attributes of the
        returned graph, rewritten by every launch."""
        return DiffGraph(self, dbatch, w, h, target, headroom)

    def device_result_to_numpy(self, r: _lib.Result, n_rasters: int) -> dict:
        out = {}
        T, N = r.n_tiles, r.n_spans

        def get(ptr, dtype, count):
            if count == 0 or not ptr:
                return np.zeros(0, dtype=dtype)
            host = np.empty(count, dtype=dtype)
            _lib.memcpy_d2h(host.ctypes.data, ptr, host.nbytes)
            return host

        out["tile_xy"] = get(r.tile_xy, np.int16, 2 * T).reshape(T, 2)
        out["tile_alpha"] = get(r.tile_alpha, np.uint8, 64 * T).reshape(T, 64)
        if r.tile_cov:
            out["tile_cov"] = get(r.tile_cov, np.float32, 64 * T).reshape(T, 64)
        out["span_xy"] = get(r.span_xy, np.int16, 2 * N).reshape(N, 2)
        out["span_w"] = get(r.span_width, np.uint16, N)
        out["span_tile"] = get(r.span_tile, np.uint32, N)
        out["raster_tile_off"] = get(r.raster_tile_off, np.uint32, n_rasters + 1).astype(np.uint64)
        out["raster_span_off"] = get(r.raster_span_off, np.uint32, n_rasters + 1).astype(np.uint64)
        return out

    @staticmethod
    def _result_to_numpy(r: _lib.Result, n_rasters: int) -> dict:
        T, N = r.n_tiles, r.n_spans
        out = {
            "tile_xy": _np_from(r.tile_xy, np.int16, 2 * T).reshape(T, 2),
            "tile_alpha": _np_from(r.tile_alpha, np.uint8, 64 * T).reshape(T, 64),
            "span_xy": _np_from(r.span_xy, np.int16, 2 * N).reshape(N, 2),
            "span_w": _np_from(r.span_width, np.uint16, N),
            "span_tile": _np_from(r.span_tile, np.uint32, N),
            "raster_tile_off": _np_from(r.raster_tile_off, np.uint32, n_rasters + 1).astype(np.uint64),
            "raster_span_off": _np_from(r.raster_span_off, np.uint32, n_rasters + 1).astype(np.uint64),
        }
        if r.tile_cov:
            out["tile_cov"] = _np_from(r.tile_cov, np.float32, 64 * T).reshape(T, 64)
        return out

    # ---- differentiable fill (device tensors as storage) ----
    def _torch_stream(self, stream: Optional[int]) -> int:
        import torch
        h = stream if stream is not None else torch.cuda.current_stream(self.device).cuda_stream
        return stream_arg(h)

    def render_coverage(self, dbatch: DeviceBatch, w: int, h: int, out=None, stream: Optional[int] = None):
        """Dense coverage images [n_rasters, h, w] (float32 CUDA tensor),
        min(|accum + area|, 1) at boundary-tile pixels, 1 in spans, else 0.
        Runs on torch's current stream unless ``stream`` is given."""
        import torch
        stream = self._torch_stream(stream)
        if out is None:
            out = torch.empty((dbatch.batch.n_rasters, h, w), dtype=torch.float32, device=f"cuda:{self.device}")
        _lib.check(_lib.load().ochre_gpu_render_coverage(self.handle, ctypes.byref(dbatch.c), w, h,
                                                         out.data_ptr(), stream), "render_coverage")
        return out

    def l2_loss(self, cov, target, dl_dcov=None, stream: Optional[int] = None):
        """(loss tensor [1] float64, dl_dcov) on the device: sum (cov - target)^2
        and, when ``dl_dcov`` is given, 2 (cov - target) written into it."""
        import torch
        stream = self._torch_stream(stream)
        loss = torch.empty(1, dtype=torch.float64, device=cov.device)
        _lib.check(_lib.load().ochre_gpu_l2_loss(self.handle, cov.data_ptr(), target.data_ptr(), cov.numel(),
                                                 loss.data_ptr(), dl_dcov.data_ptr() if dl_dcov is not None else None,
                                                 stream), "l2_loss")
        return loss, dl_dcov

    def fill_backward(self, dbatch: DeviceBatch, w: int, h: int, dl_dcov, dl_dpts=None, dl_dxf=None,
                      stream: Optional[int] = None):
        """dL/d(points) [n_floats] and dL/d(transforms) [n_fills, 6] (CUDA tensors)
        from dL/d(coverage) [n_rasters, h, w]."""
        import torch
        stream = self._torch_stream(stream)
        dev = dl_dcov.device
        if dl_dpts is None:
            dl_dpts = torch.empty(max(1, len(dbatch.batch.pts)), dtype=torch.float32, device=dev)
        if dl_dxf is None:
            dl_dxf = torch.empty((max(1, dbatch.batch.n_fills), 6), dtype=torch.float32, device=dev)
        _lib.check(_lib.load().ochre_gpu_fill_backward(self.handle, ctypes.byref(dbatch.c), w, h,
                                                       dl_dcov.data_ptr(), dl_dpts.data_ptr(), dl_dxf.data_ptr(),
                                                       stream), "fill_backward")
        return dl_dpts, dl_dxf

    def composite(self, result: _lib.Result, n_rasters: int, colors, canvas, stream: Optional[int] = None):
        """Draw the rasters of a device result (rasterize_device) onto an RGBA8
        canvas (uint8 CUDA tensor [h, w, 4], updated in place) with one RGBA8
        colour per raster (uint8 CUDA tensor [n_rasters, 4]), in raster order:
        the reference example's tile/span quads, colour * mask, blended
        SRC_ALPHA / ONE_MINUS_SRC_ALPHA, quantised after every quad."""
        stream = self._torch_stream(stream)
        h, w = int(canvas.shape[0]), int(canvas.shape[1])
        _lib.check(_lib.load().ochre_gpu_composite(self.handle, ctypes.byref(result), n_rasters, colors.data_ptr(),
                                                   w, h, canvas.data_ptr(), stream), "composite")
        return canvas

    def stats(self) -> dict:
        s = _lib.Stats()
        _lib.check(_lib.load().ochre_gpu_last_stats(self.handle, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in _lib.Stats._fields_ if not k.startswith("pad")}
