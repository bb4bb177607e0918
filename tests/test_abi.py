"""CPU tests of the C-ABI library: it builds for sm_103a, loads, and exports
every entry point include/ochre_gpu.h declares (no compute without a GPU)."""
import ctypes
import os
import re

import pytest

from ochre_gb300 import _lib, build
from ochre_gb300 import batch as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            src = re.sub(r"//[^\n]*", "", src)
            names |= set(re.findall(r"\b(ochre_\w+)\s*\(", src))
    return {n for n in names if not n.endswith("_fn")}


def test_library_builds_and_exports_every_declared_symbol():
    path = build.build()
    assert os.path.exists(path)
    lib = ctypes.CDLL(path)
    declared = _declared()
    assert "ochre_gpu_rasterize" in declared and "ochre_rasterizer_finish" in declared
    missing = [n for n in sorted(declared) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_lib.EXPORTS) <= declared


def test_status_strings_without_gpu():
    assert _lib.status_string(_lib.OK) == "ok"
    assert "invalid" in _lib.status_string(_lib.E_INVALID)


def test_header_constants_match_python():
    src = open(os.path.join(ROOT, "include", "ochre_gpu.h")).read()
    for name, val in [("OCHRE_MOVE", B.MOVE), ("OCHRE_LINE", B.LINE), ("OCHRE_QUADRATIC", B.QUADRATIC),
                      ("OCHRE_CUBIC", B.CUBIC), ("OCHRE_CONIC", B.CONIC), ("OCHRE_CLOSE", B.CLOSE)]:
        assert re.search(rf"{name}\s*=\s*{val}\b", src), name
    assert re.search(r"OCHRE_FILL_RAW\s+1u", src)
    assert re.search(r"OCHRE_TILE_SIZE\s+8\b", src)


def test_create_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from ochre_gb300 import GpuContext
    with pytest.raises(_lib.OchreError):
        GpuContext(0)


def test_validate_batch_checks_the_structure():
    """ochre_validate_batch (host only): offset arrays must start at 0, not
    decrease and end at the counts; the check ochre_gpu_rasterize makes."""
    import dataclasses

    import numpy as np

    from ochre_gb300 import OchreError, validate_batch
    from ochre_gb300 import workloads as W
    b = W.glyph_run(n_paths=300, seed=4)
    validate_batch(b)
    bad_cases = []
    off = b.fill_cmd_off.copy()
    off[10], off[11] = off[11], off[10]            # decreasing
    bad_cases.append(dataclasses.replace(b, fill_cmd_off=off))
    off = b.fill_cmd_off.copy()
    off[-1] -= 1                                    # does not end at n_cmds
    bad_cases.append(dataclasses.replace(b, fill_cmd_off=off))
    off = b.fill_cmd_off.copy()
    off[0] = 1                                      # does not start at 0
    bad_cases.append(dataclasses.replace(b, fill_cmd_off=off))
    roff = np.arange(b.n_rasters + 1, dtype=np.uint32)
    roff[5], roff[6] = roff[6], roff[5]
    bad_cases.append(dataclasses.replace(b, raster_fill_off=roff))
    bad_cases.append(dataclasses.replace(b, raster_fill_off=None, n_rasters=b.n_rasters - 1))
    for bad in bad_cases:
        with pytest.raises(OchreError) as e:
            validate_batch(bad)
        assert e.value.status == _lib.E_INVALID
    # a raster holding several fills, and an empty batch
    validate_batch(dataclasses.replace(b, raster_fill_off=np.array([0, 100, b.n_fills], np.uint32), n_rasters=2))
    from ochre_gb300 import BatchBuilder
    validate_batch(BatchBuilder().build())


def test_struct_layouts_match_the_header(tmp_path):
    """The ctypes structures (sizes and field offsets) are the header's C
    structures, compiled here with the host C compiler."""
    import ctypes
    import os
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = [("ochre_batch", _lib.Batch), ("ochre_result", _lib.Result), ("ochre_stats", _lib.Stats),
             ("ochre_kernel_time", _lib.KernelTime), ("ochre_output_buffers", _lib.OutputBuffers)]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ochre_gpu.h"', "int main(void) {"]
    for cname, cls in pairs:
        lines.append(f'    printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'    printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")
    subprocess.run([cc, "-std=c11", "-I", inc, str(src), "-o", str(exe)], check=True)
    got = dict(line.rsplit(" ", 1) for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                              text=True).stdout.splitlines())
    for cname, cls in pairs:
        assert int(got[cname]) == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(cls, fname).offset, (cname, fname)
