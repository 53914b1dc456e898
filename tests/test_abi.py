"""The C-ABI library loads and exports every symbol include/shapes_gpu.h
declares (no compute calls: runs without a GPU)."""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    text = (ROOT / "include" / "shapes_gpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(shapes_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for must in ("shapes_batch_create", "shapes_batch_step", "shapes_batch_collide", "shapes_batch_get_bodies",
                 "shapes_batch_get_cache", "shapes_batch_set_cache", "shapes_batch_destroy", "shapes_strerror"):
        assert must in syms


def test_library_exports_all_declared_symbols(built):
    from shapes_gb300 import _lib

    handle = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [s for s in declared_symbols() if not hasattr(handle, s)]
    assert not missing, missing
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(declared_symbols()) <= bound


def test_strerror_and_argument_errors(built):
    from shapes_gb300 import _lib

    L = _lib.lib()
    assert L.shapes_strerror(0) == b"ok"
    assert L.shapes_strerror(-3).startswith(b"hull")
    # argument validation happens before any device work
    h = ctypes.c_void_p()
    assert L.shapes_batch_create(0, None, None, None, None, None, ctypes.byref(h)) == _lib.SHAPES_E_INVALID_ARG
    assert L.shapes_batch_step(None, None, 1) == _lib.SHAPES_E_INVALID_ARG
    # the multi-handle entry points refuse missing handles, counts and buffers
    cfg = _lib.make_config(1.0 / 60.0)
    none = (ctypes.c_void_p * 1)(None)
    bodies = (_lib.Bodies * 1)()
    assert L.shapes_batches_step(None, 1, ctypes.byref(cfg), 1) == _lib.SHAPES_E_INVALID_ARG
    assert L.shapes_batches_step_io(none, 1, ctypes.byref(cfg), bodies, bodies) == _lib.SHAPES_E_INVALID_ARG
    assert L.shapes_batches_run_io(none, 0, ctypes.byref(cfg), 1, bodies, _lib.STEP_CALLBACK(),
                                   None) == _lib.SHAPES_E_INVALID_ARG
    assert L.shapes_batches_run_io(none, 1, ctypes.byref(cfg), -1, bodies, _lib.STEP_CALLBACK(),
                                   None) == _lib.SHAPES_E_INVALID_ARG
    assert L.shapes_batches_run_io(none, 1, ctypes.byref(cfg), 1, bodies, _lib.STEP_CALLBACK(),
                                   None) == _lib.SHAPES_E_INVALID_ARG
    # per-handle options refuse a missing handle
    assert L.shapes_batch_set_narrowphase_lanes(None, 32) == _lib.SHAPES_E_INVALID_ARG
    assert L.shapes_batch_set_wait_limit(None, 1) == _lib.SHAPES_E_INVALID_ARG
    assert L.shapes_batch_set_sweep_prune(None, 1) == _lib.SHAPES_E_INVALID_ARG
    v = ctypes.c_int32()
    assert L.shapes_batch_get_group_target(None, ctypes.byref(v)) == _lib.SHAPES_E_INVALID_ARG


def test_product_does_not_import_oracle():
    for p in (ROOT / "shapes_gb300").rglob("*.py"):
        assert "oracle" not in re.findall(r"^\s*(?:from|import)\s+(\w+)", p.read_text(), flags=re.M), p
    for p in (ROOT / "shapes_gb300" / "csrc").rglob("*"):
        if p.suffix in (".cu", ".cuh", ".h"):
            includes = re.findall(r'^\s*#\s*include\s*[<"]([^>"]+)', p.read_text(), flags=re.M)
            assert not any("oracle" in inc for inc in includes), p
