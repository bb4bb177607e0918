"""Host-side input layout shared by the C-ABI (``ochre_batch`` in
include/ochre_gpu.h), the Python mirror and the tests.

A *raster* is one ochre ``Rasterizer``: ``Rasterizer::new()``, one or more
``fill(&[PathCmd], Transform)`` calls, then ``finish`` (src/rasterizer.rs:50,
161, 180).  A *fill* is one ``fill`` call: a run of commands plus its
transform.  Commands are flattened from ochre's ``PathCmd`` enum
(src/path.rs:5-12), which is not ``repr(C)``, into a verb byte plus a float
stream:

=========  ====  =========================================
verb       code  floats (in order)
=========  ====  =========================================
Move       0     x y
Line       1     x y
Quadratic  2     cx cy x y
Cubic      3     c1x c1y c2x c2y x y
Conic      4     cx cy x y w
Close      5     (none)
=========  ====  =========================================

A transform is ``m0 m1 m2 m3 ox oy``: the row-major ``Mat2x2`` and offset of
``Transform`` (src/geom.rs:133, 204-207).  Fills flagged ``RAW`` are not
transformed (``Rasterizer::command`` / ``move_to`` / ``line_to`` take points
in device space, src/rasterizer.rs:61, 72, 145).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Iterable, Optional, Sequence

import numpy as np

MOVE, LINE, QUADRATIC, CUBIC, CONIC, CLOSE = 0, 1, 2, 3, 4, 5
FLOATS_PER_VERB = np.array([2, 2, 4, 6, 5, 0], dtype=np.int64)
FILL_RAW = 1
FILL_STROKE = 2

IDENTITY = np.array([1.0, 0.0, 0.0, 1.0, 0.0, 0.0], dtype=np.float32)


@dataclass
class Batch:
    verbs: np.ndarray                       # uint8 [n_cmds]
    pts: np.ndarray                         # float32 [n_floats]
    fill_cmd_off: np.ndarray                # uint32 [n_fills + 1]
    fill_xf: np.ndarray                     # float32 [n_fills, 6]
    fill_flags: Optional[np.ndarray]        # uint8 [n_fills] or None
    raster_fill_off: Optional[np.ndarray]   # uint32 [n_rasters + 1] or None (one fill per raster)
    n_rasters: int
    fill_width: Optional[np.ndarray] = None # float32 [n_fills]: stroke width where flags & FILL_STROKE

    @property
    def n_cmds(self) -> int:
        return int(len(self.verbs))

    @property
    def n_fills(self) -> int:
        return int(len(self.fill_cmd_off) - 1)

    def input_bytes(self) -> int:
        """Compulsory input bytes: 1 per verb, 4 per float, 24 per transform."""
        return int(self.verbs.nbytes + self.pts.nbytes + 24 * self.n_fills)

    @property
    def has_strokes(self) -> bool:
        return self.fill_flags is not None and bool(np.any(self.fill_flags & FILL_STROKE))

    def validate(self) -> None:
        v = self.verbs
        if v.dtype != np.uint8 or (len(v) and int(v.max()) > CLOSE):
            raise ValueError("verbs must be uint8 codes 0..5")
        need = int(FLOATS_PER_VERB[v].sum()) if len(v) else 0
        if need > len(self.pts):
            raise ValueError(f"point stream too short: need {need} floats, have {len(self.pts)}")
        off = self.fill_cmd_off
        if off[0] != 0 or off[-1] != len(v) or np.any(np.diff(off.astype(np.int64)) < 0):
            raise ValueError("fill_cmd_off must start at 0, end at n_cmds and be non-decreasing")
        if self.fill_xf.shape != (self.n_fills, 6):
            raise ValueError("fill_xf must be [n_fills, 6]")
        if self.has_strokes and (self.fill_width is None or len(self.fill_width) != self.n_fills):
            raise ValueError("stroked fills need fill_width [n_fills]")
        if self.raster_fill_off is None:
            if self.n_rasters != self.n_fills:
                raise ValueError("without raster_fill_off there is one fill per raster")
        else:
            r = self.raster_fill_off
            if len(r) != self.n_rasters + 1 or r[0] != 0 or r[-1] != self.n_fills or np.any(np.diff(r.astype(np.int64)) < 0):
                raise ValueError("raster_fill_off must have n_rasters+1 non-decreasing entries from 0 to n_fills")


class BatchBuilder:
    """Accumulates rasters/fills/commands into a :class:`Batch`."""

    def __init__(self) -> None:
        self._verbs: list[np.ndarray] = []
        self._pts: list[np.ndarray] = []
        self._fill_ncmd: list[int] = []
        self._xf: list[np.ndarray] = []
        self._flags: list[int] = []
        self._width: list[float] = []
        self._raster_nfill: list[int] = []

    def begin_raster(self) -> "BatchBuilder":
        self._raster_nfill.append(0)
        return self

    def fill(self, verbs: Sequence[int] | np.ndarray, pts: Sequence[float] | np.ndarray,
             transform: Optional[Iterable[float]] = None, raw: bool = False,
             stroke_width: Optional[float] = None) -> "BatchBuilder":
        """Rasterizer::fill (or Rasterizer::stroke when ``stroke_width`` is set)."""
        if not self._raster_nfill:
            self.begin_raster()
        v = np.asarray(verbs, dtype=np.uint8).reshape(-1)
        p = np.asarray(pts, dtype=np.float32).reshape(-1)
        self._verbs.append(v)
        self._pts.append(p)
        self._fill_ncmd.append(len(v))
        xf = IDENTITY if transform is None else np.asarray(list(transform), dtype=np.float32).reshape(6)
        self._xf.append(xf)
        self._flags.append((FILL_RAW if raw else 0) | (FILL_STROKE if stroke_width is not None else 0))
        self._width.append(0.0 if stroke_width is None else float(stroke_width))
        self._raster_nfill[-1] += 1
        return self

    def build(self) -> Batch:
        verbs = np.concatenate(self._verbs) if self._verbs else np.zeros(0, np.uint8)
        pts = np.concatenate(self._pts) if self._pts else np.zeros(0, np.float32)
        off = np.zeros(len(self._fill_ncmd) + 1, dtype=np.uint32)
        if self._fill_ncmd:
            off[1:] = np.cumsum(self._fill_ncmd)
        xf = np.stack(self._xf).astype(np.float32) if self._xf else np.zeros((0, 6), np.float32)
        flags = np.asarray(self._flags, dtype=np.uint8)
        roff = np.zeros(len(self._raster_nfill) + 1, dtype=np.uint32)
        if self._raster_nfill:
            roff[1:] = np.cumsum(self._raster_nfill)
        width = np.asarray(self._width, dtype=np.float32) if np.any(flags & FILL_STROKE) else None
        b = Batch(verbs, pts, off, xf, flags if np.any(flags) else None, roff, len(self._raster_nfill), width)
        b.validate()
        return b


def concat(batches: Sequence[Batch]) -> Batch:
    """Concatenate batches raster-wise."""
    verbs = np.concatenate([b.verbs for b in batches])
    pts = np.concatenate([b.pts for b in batches])
    offs, xfs, flags, roffs = [], [], [], []
    cbase = fbase = 0
    for b in batches:
        offs.append(b.fill_cmd_off[:-1].astype(np.int64) + cbase)
        xfs.append(b.fill_xf)
        flags.append(b.fill_flags if b.fill_flags is not None else np.zeros(b.n_fills, np.uint8))
        rf = b.raster_fill_off if b.raster_fill_off is not None else np.arange(b.n_fills + 1, dtype=np.uint32)
        roffs.append(rf[:-1].astype(np.int64) + fbase)
        cbase += b.n_cmds
        fbase += b.n_fills
    off = np.concatenate(offs + [np.array([cbase])]).astype(np.uint32)
    roff = np.concatenate(roffs + [np.array([fbase])]).astype(np.uint32)
    fl = np.concatenate(flags).astype(np.uint8)
    width = None
    if any(b.fill_width is not None for b in batches):
        width = np.concatenate([b.fill_width if b.fill_width is not None else np.zeros(b.n_fills, np.float32)
                                for b in batches]).astype(np.float32)
    out = Batch(verbs, pts, off, np.concatenate(xfs).astype(np.float32),
                fl if np.any(fl) else None, roff, sum(b.n_rasters for b in batches), width)
    out.validate()
    return out


def subset(b: Batch, rasters: Sequence[int]) -> Batch:
    """A batch holding only the given rasters (in the given order)."""
    roff = b.raster_fill_off if b.raster_fill_off is not None else np.arange(b.n_fills + 1, dtype=np.uint32)
    fpo = np.concatenate([[0], np.cumsum(FLOATS_PER_VERB[b.verbs])]).astype(np.int64)
    bb = BatchBuilder()
    for r in rasters:
        bb.begin_raster()
        for f in range(int(roff[r]), int(roff[r + 1])):
            c0, c1 = int(b.fill_cmd_off[f]), int(b.fill_cmd_off[f + 1])
            raw = b.fill_flags is not None and bool(b.fill_flags[f] & FILL_RAW)
            stroke = b.fill_flags is not None and bool(b.fill_flags[f] & FILL_STROKE)
            bb.fill(b.verbs[c0:c1], b.pts[fpo[c0]:fpo[c1]], b.fill_xf[f], raw=raw,
                    stroke_width=float(b.fill_width[f]) if stroke else None)
    return bb.build()
