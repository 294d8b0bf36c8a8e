"""The C ABI library loads without a GPU, exports every symbol include/edgpu.h declares, and rejects
bad arguments with the reference's error classes before touching a device.  No compute call here."""
import ctypes
import os
import re
import subprocess
import sys

import numpy as np
import pytest

import edgpu
from edgpu import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "edgpu.h")).read()
    return sorted(set(re.findall(r"^(?:int|void|const char\*)\s+(edgpu_\w+)\s*\(", src, re.M)))


def test_every_declared_symbol_is_exported_and_bound():
    L = _lib.lib()
    syms = declared_symbols()
    assert len(syms) >= 30
    for s in syms:
        assert hasattr(L, s), s
        assert s in _lib.SIGNATURES, f"{s} has no ctypes signature"


def test_version_and_device_count_without_gpu():
    assert b"sm_103a" in _lib.lib().edgpu_version()
    assert _lib.device_count() >= 0


def test_argument_errors_before_device():
    L = _lib.lib()
    h = ctypes.c_void_p()
    dims = np.full(64, 2, dtype=np.int32)
    qn = np.tile(np.array([1, -1], dtype=np.int64), 64)
    al = np.array([0], dtype=np.int64)
    st = L.edgpu_space_create(64, _lib.ptr(dims, ctypes.c_int32), 1, _lib.ptr(qn, ctypes.c_int64), 1,
                              _lib.ptr(al, ctypes.c_int64), 0, ctypes.byref(h))
    assert st == _lib.ERR_ARG and b"not enough" in L.edgpu_last_error()
    st = L.edgpu_space_create(0, _lib.ptr(dims, ctypes.c_int32), 1, None, 0, None, 0, ctypes.byref(h))
    assert st == _lib.ERR_ARG
    assert L.edgpu_op_create(None, 0, None, None, None, None, None, 0, None, ctypes.byref(h)) == _lib.ERR_ARG
    assert L.edgpu_mul(None, 0, None, None, 0, 0) == _lib.ERR_ARG
    assert L.edgpu_reduce(None, 1, None, None, None, 1, ctypes.byref(h)) == _lib.ERR_ARG
    # the slab table's entry points: null handles are refused before any device work
    cur = ctypes.c_int32()
    assert L.edgpu_op_slab_scaling(None, 2, ctypes.byref(cur)) == _lib.ERR_ARG
    assert L.edgpu_op_slab_use(None, 0, 1, ctypes.byref(cur)) == _lib.ERR_ARG
    assert L.edgpu_op_build_slabs(None, 1 << 20, 0, ctypes.byref(cur)) == _lib.ERR_ARG
    assert L.edgpu_op_free_slabs(None) == _lib.ERR_ARG
    with pytest.raises(edgpu.ArgumentError):
        _lib.check(_lib.ERR_ARG)
    with pytest.raises(edgpu.DimensionMismatch):
        _lib.check(_lib.ERR_DIM)


def test_package_fails_loudly_without_library(tmp_path):
    pkg = os.path.join(ROOT, "exactdiagonalization.jl_gb300", "edgpu")
    dst = tmp_path / "edgpu"
    dst.mkdir()
    for f in os.listdir(pkg):
        if f.endswith(".py"):
            (dst / f).write_text(open(os.path.join(pkg, f)).read())
    r = subprocess.run([sys.executable, "-c", "import edgpu"], cwd=tmp_path, capture_output=True, text=True)
    assert r.returncode != 0 and "libedgpu.so is not built" in r.stderr
