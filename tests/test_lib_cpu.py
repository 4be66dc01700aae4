"""CPU-side checks of the GPU library: it builds for sm_103a, loads, and exports
every entry point declared in include/alfgpu.h.  No compute calls (no GPU here)."""
import ctypes

from alf_gb300 import _lib, build


def test_library_builds_and_exports_header_symbols():
    path = build.build()
    L = ctypes.CDLL(path)
    names = _lib.header_functions()
    assert "alfgpu_sweep" in names and "alfgpu_init_state" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_error_strings_without_gpu():
    L = _lib.lib()
    assert L.alfgpu_error_string(3) == b"Precision Green exceeds 10: unstable calculation"
    assert L.alfgpu_error_string(0) == b"no error"


def test_create_rejects_bad_dims_before_touching_the_device():
    L = _lib.lib()
    h = ctypes.c_void_p()
    d = _lib.Dims(0, 2, 1, 16, 40, 10, 1, 0, 0, 0, 0)
    assert L.alfgpu_create(ctypes.byref(h), ctypes.byref(d)) == 101
    d = _lib.Dims(16, 3, 1, 16, 40, 10, 1, 0, 0, 0, 0)
    assert L.alfgpu_create(ctypes.byref(h), ctypes.byref(d)) == 101
