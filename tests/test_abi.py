"""CPU: the C ABI library loads, exports every declared symbol, and rejects
bad arguments on the host before touching a device."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for fn in os.listdir(inc):
        if fn.endswith(".h"):
            src = open(os.path.join(inc, fn)).read()
            names |= set(re.findall(r"HGB_API\s+[\w\s\*]*?\b(hgb_\w+)\s*\(", src))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("hgb_local_op", "hgb_sobel_mag", "hgb_point_gray", "hgb_reduce", "hgb_separable", "hgb_bilateral",
                 "hgb_pyramid_decompose", "hgb_local_op_adjoint", "hgb_conv_bilateral_mse", "hgb_init"):
        assert must in names


def test_library_exports_every_declared_symbol(hgb_lib):
    from hipacc_gb300 import _lib

    missing = [n for n in declared_symbols() if not hasattr(hgb_lib, n)]
    assert not missing, missing
    # and the Python binding covers them all
    assert declared_symbols() <= set(_lib.SIGNATURES)


def test_abi_version(hgb_lib):
    assert hgb_lib.hgb_abi_version() == 1


def test_host_side_validation_without_gpu(hgb_lib):
    """Invalid requests fail with HGB_ERR_INVALID and a message, no device call."""
    from hipacc_gb300 import _lib as L

    rc = hgb_lib.hgb_local_op(None, None, None, None, None, None, None, 3, 3, 0, 1, 0.0, None)
    assert rc == L.ERR_INVALID
    assert b"null view" in hgb_lib.hgb_last_error()
    v = L.View(0x1000, L.F32, 16, 16, 1, 64, 1024)
    bad = L.View(0x1000, L.F32, 16, 16, 1, 32, 1024)  # pitch below a row
    rc = hgb_lib.hgb_local_op(C.byref(v), None, C.byref(bad), None, None, None, None, 3, 3, 0, 1, 0.0, None)
    assert rc == L.ERR_INVALID and b"pitch" in hgb_lib.hgb_last_error()
    rc = hgb_lib.hgb_local_op(C.byref(v), None, C.byref(v), None, None, None, None, 17, 3, 0, 1, 0.0, None)
    assert rc == L.ERR_INVALID and b"mask size" in hgb_lib.hgb_last_error()
    w = L.Window(10, 10, 10, 10)  # outside a 16x16 image
    m = (C.c_float * 9)()
    rc = hgb_lib.hgb_local_op(C.byref(v), C.byref(w), C.byref(v), None, m, None, None, 3, 3, 0, 1, 0.0, None)
    assert rc == L.ERR_INVALID and b"window" in hgb_lib.hgb_last_error()
    u8 = L.View(0x1000, L.U8, 16, 16, 1, 16, 256)
    rc = hgb_lib.hgb_sobel_mag(C.byref(u8), C.byref(u8), None, None, 3, 3, 0, None, None, None)
    assert rc == L.ERR_INVALID
    rc = hgb_lib.hgb_point_gray(C.byref(u8), C.byref(u8), 77, 150, 29, 8, None)
    assert rc == L.ERR_INVALID and b"uchar4" in hgb_lib.hgb_last_error()
    rc = hgb_lib.hgb_reduce(C.byref(u8), None, 7, None, None, None)
    assert rc == L.ERR_INVALID


def test_validation_of_storage_and_operator_arguments(hgb_lib):
    """Storage pairs, histogram, bilateral and resampling arguments are checked on the host."""
    from hipacc_gb300 import _lib as L

    u8 = L.View(0x1000, L.U8, 16, 16, 1, 16, 256)
    bf = L.View(0x1000, L.BF16, 16, 16, 1, 32, 512)
    f32 = L.View(0x1000, L.F32, 16, 16, 1, 64, 1024)
    m = (C.c_float * 9)()
    # u8 output only from u8 input
    rc = hgb_lib.hgb_local_op(C.byref(bf), None, C.byref(u8), None, m, None, None, 3, 3, 0, 1, 0.0, None)
    assert rc == L.ERR_INVALID and b"u8" in hgb_lib.hgb_last_error()
    # histogram: bin count and result buffer
    rc = hgb_lib.hgb_histogram(C.byref(u8), None, 0, C.c_void_p(0x2000), None, None)
    assert rc == L.ERR_INVALID and b"num_bins" in hgb_lib.hgb_last_error()
    rc = hgb_lib.hgb_histogram(C.byref(u8), None, 16385, C.c_void_p(0x2000), None, None)
    assert rc == L.ERR_INVALID and b"num_bins" in hgb_lib.hgb_last_error()
    rc = hgb_lib.hgb_histogram(C.byref(u8), None, 256, None, None, None)
    assert rc == L.ERR_INVALID and b"result" in hgb_lib.hgb_last_error()
    rc = hgb_lib.hgb_histogram(C.byref(bf), None, 256, C.c_void_p(0x2000), None, None)
    assert rc == L.ERR_INVALID
    # bilateral: odd sizes 3..13, positive sigma, non-negative weights, same storage
    sm = (C.c_float * 169)(*([0.5] * 169))
    for size, sigma in ((4, 0.1), (15, 0.1), (5, 0.0)):
        rc = hgb_lib.hgb_bilateral(C.byref(f32), C.byref(f32), sm, size, sigma, 1, 0.0, 0, None)
        assert rc == L.ERR_INVALID, (size, sigma)
    rc = hgb_lib.hgb_bilateral(C.byref(f32), C.byref(bf), sm, 5, 0.1, 1, 0.0, 0, None)
    assert rc == L.ERR_INVALID
    neg = (C.c_float * 9)(*([0.5] * 8 + [-1.0]))
    rc = hgb_lib.hgb_bilateral(C.byref(f32), C.byref(f32), neg, 3, 0.1, 1, 0.0, 0, None)
    assert rc == L.ERR_INVALID and b"non-negative" in hgb_lib.hgb_last_error()
    # packed half weights need half storage
    rc = hgb_lib.hgb_bilateral(C.byref(f32), C.byref(f32), sm, 5, 0.1, 1, 0.0, 1, None)
    assert rc == L.ERR_INVALID
    # resampling modes 1..5 only
    for mode in (0, 6):
        rc = hgb_lib.hgb_resample(C.byref(f32), C.byref(f32), mode, None)
        assert rc == L.ERR_INVALID and b"imode" in hgb_lib.hgb_last_error()


def test_autotune_cache_persistence(hgb_lib, tmp_path):
    """The tile-configuration cache round-trips through its JSON file (host only)."""
    from hipacc_gb300 import _lib as L

    src = tmp_path / "tune.json"
    src.write_text('{\n  "conv|f32|5x5|1024x1024": [1, 0.084000],\n  "conv|u8|5x5|1024x1024": [2, 0.120000]\n}\n')
    assert hgb_lib.hgb_autotune_clear() == L.OK
    assert hgb_lib.hgb_autotune_count() == 0
    assert hgb_lib.hgb_autotune_load(str(src).encode()) == L.OK
    assert hgb_lib.hgb_autotune_count() == 2
    out = tmp_path / "saved.json"
    assert hgb_lib.hgb_autotune_save(str(out).encode()) == L.OK
    assert hgb_lib.hgb_autotune_clear() == L.OK and hgb_lib.hgb_autotune_count() == 0
    assert hgb_lib.hgb_autotune_load(str(out).encode()) == L.OK
    assert hgb_lib.hgb_autotune_count() == 2
    text = out.read_text()
    assert '"conv|u8|5x5|1024x1024": [2, 0.120000]' in text
    bad = tmp_path / "bad.json"
    bad.write_text('{"key": "no configuration here"}')
    assert hgb_lib.hgb_autotune_load(str(bad).encode()) == L.ERR_INVALID
    assert hgb_lib.hgb_autotune_load(str(tmp_path / "missing.json").encode()) == L.ERR_INVALID
    assert hgb_lib.hgb_autotune_save(None) == L.ERR_INVALID
    assert hgb_lib.hgb_autotune_clear() == L.OK


def test_python_api_rejects_host_tensors(hgb_lib):
    """The torch binding refuses CPU tensors instead of passing host pointers to the kernels."""
    import numpy as np
    import torch

    from hipacc_gb300 import api

    x = torch.zeros((8, 8))
    with pytest.raises(ValueError, match="CUDA tensors"):
        api.local_op(x, torch.zeros_like(x), mask=np.ones((3, 3), np.float32))
    with pytest.raises(ValueError, match="CUDA tensors"):
        api.histogram(torch.zeros((8, 8), dtype=torch.uint8), 16)


def test_missing_library_fails_loudly(tmp_path):
    from hipacc_gb300 import _lib as L

    saved = L._lib
    L._lib = None
    try:
        with pytest.raises(RuntimeError, match="no fallback"):
            L.load(str(tmp_path / "nope.so"))
    finally:
        L._lib = saved


def test_samples_compile_and_link(hgb_lib, tmp_path):
    """The C++ host surface compiles and links against the library (CPU only)."""
    import subprocess

    lib = os.path.join(ROOT, "hipacc_gb300")
    for name in ("gaussian_blur", "sobel", "color_reduce", "pyramid", "bilateral", "graph"):
        r = subprocess.run(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "include"),
                            os.path.join(ROOT, "tests", "samples", name + ".cpp"), "-L", lib, "-lhipacc_gb300",
                            "-Wl,-rpath," + lib, "-o", str(tmp_path / name)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
