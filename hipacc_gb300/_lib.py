"""ctypes binding of libhipacc_gb300.so (the C ABI in include/hipacc_gb300.h).

The shared library is built in-tree by ``hipacc_gb300.build``.  Loading fails
loudly when it is missing: there is no CPU fallback anywhere in this package.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libhipacc_gb300.so")

# hgb_status
OK, ERR_INVALID, ERR_UNSUPPORTED, ERR_CUDA, ERR_ALLOC, ERR_TIMEOUT, ERR_LIMIT, ERR_INTERNAL = range(8)
# hgb_dtype
U8, U8X4, I16, U16, I32, U32, U64, F16, BF16, F32, F64 = range(11)
DTYPE_SIZE = {U8: 1, U8X4: 4, I16: 2, U16: 2, I32: 4, U32: 4, U64: 8, F16: 2, BF16: 2, F32: 4, F64: 8}
# hipacc::Boundary / hipacc::Reduce numbering
UNDEFINED, CLAMP, REPEAT, MIRROR, CONSTANT = range(5)
SUM, MIN, MAX, PROD = range(4)


class HgbError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"hipacc_gb300 status {status}: {msg}")
        self.status = status


class View(C.Structure):
    _fields_ = [("data", C.c_void_p), ("dtype", C.c_int32), ("width", C.c_int32), ("height", C.c_int32),
                ("batch", C.c_int32), ("pitch", C.c_int64), ("batch_stride", C.c_int64)]


class Window(C.Structure):
    _fields_ = [("offset_x", C.c_int32), ("offset_y", C.c_int32), ("width", C.c_int32), ("height", C.c_int32)]


VP = C.POINTER(View)
WP = C.POINTER(Window)
vp = C.c_void_p
i32 = C.c_int
f32 = C.c_float

# name -> (restype, argtypes); every function of the header
SIGNATURES = {
    "hgb_abi_version": (i32, []),
    "hgb_init": (i32, [i32, C.c_char_p, C.c_size_t]),
    "hgb_last_error": (C.c_char_p, []),
    "hgb_set_timing": (i32, [i32]),
    "hgb_last_kernel_timing": (f32, []),
    "hgb_autotune_enable": (i32, [i32]),
    "hgb_autotune_clear": (i32, []),
    "hgb_autotune_count": (i32, []),
    "hgb_autotune_save": (i32, [C.c_char_p]),
    "hgb_autotune_load": (i32, [C.c_char_p]),
    "hgb_workspace_reserve": (i32, [C.c_size_t]),
    "hgb_device_status": (i32, [C.POINTER(C.c_int)]),
    "hgb_image_create": (i32, [i32, i32, i32, i32, vp, C.POINTER(vp)]),
    "hgb_image_destroy": (i32, [vp]),
    "hgb_image_get_view": (i32, [vp, VP]),
    "hgb_image_write": (i32, [vp, vp, vp]),
    "hgb_image_read": (i32, [vp, vp, vp]),
    "hgb_image_read_async": (i32, [vp, vp, vp]),
    "hgb_histogram": (i32, [vp, vp, C.c_uint, vp, vp, vp]),
    "hgb_stream_create": (i32, [vp]),
    "hgb_stream_destroy": (i32, [vp]),
    "hgb_stream_synchronize": (i32, [vp]),
    "hgb_stream_wait": (i32, [vp, vp]),
    "hgb_graph_begin": (i32, [vp]),
    "hgb_graph_end": (i32, [vp, vp]),
    "hgb_graph_launch": (i32, [vp, vp]),
    "hgb_graph_destroy": (i32, [vp]),
    "hgb_image_copy": (i32, [vp, vp, vp]),
    "hgb_image_copy_region": (i32, [vp, WP, vp, WP, vp]),
    "hgb_local_op": (i32, [VP, WP, VP, WP, vp, vp, vp, i32, i32, i32, i32, f32, vp]),
    "hgb_separable": (i32, [VP, VP, vp, vp, i32, i32, f32, vp]),
    "hgb_bilateral": (i32, [VP, VP, vp, i32, f32, i32, f32, i32, vp]),
    "hgb_sobel_mag": (i32, [VP, VP, vp, vp, i32, i32, i32, vp, vp, vp]),
    "hgb_point_gray": (i32, [VP, VP, i32, i32, i32, i32, vp]),
    "hgb_point_binary": (i32, [i32, VP, VP, VP, f32, f32, vp]),
    "hgb_convert": (i32, [VP, VP, vp]),
    "hgb_resample": (i32, [VP, VP, i32, vp]),
    "hgb_harris_corner": (i32, [VP, VP, f32, f32, i32, i32, vp]),
    "hgb_unsharp": (i32, [VP, VP, i32, i32, vp]),
    "hgb_reduce": (i32, [VP, WP, i32, vp, vp, vp]),
    "hgb_reduce_noalloc": (i32, [VP, WP, i32, vp, vp, vp]),
    "hgb_pyramid_plan_create": (i32, [i32, vp, vp, i32, vp, i32, C.POINTER(vp)]),
    "hgb_pyramid_plan_destroy": (i32, [vp]),
    "hgb_pyramid_level_view": (i32, [vp, i32, i32, VP, VP]),
    "hgb_pyramid_decompose": (i32, [vp, i32, vp]),
    "hgb_pyramid_collapse": (i32, [vp, vp]),
    "hgb_pyramid_plan_wait_test": (i32, [vp, C.c_longlong, i32, i32]),
    "hgb_pyramid_plan_trace": (i32, [vp, vp, C.c_longlong]),
    "hgb_local_op_adjoint": (i32, [VP, VP, VP, vp, vp, i32, i32, i32, vp, vp]),
    "hgb_bilateral_adjoint": (i32, [VP, VP, vp, i32, f32, i32, f32, VP, vp, vp]),
    "hgb_separable_adjoint": (i32, [VP, VP, vp, vp, i32, i32, f32, VP, vp, vp, vp]),
    "hgb_local_op_minmax_adjoint": (i32, [VP, VP, VP, vp, vp, i32, i32, i32, i32, f32, vp]),
    "hgb_conv_bilateral_mse": (i32, [VP, VP, vp, i32, vp, i32, vp, i32, i32, vp, VP, vp, vp, vp]),
}

_lib = None


def load(path: str | None = None):
    """Load the library (once).  Raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with hipacc_gb300.build.build() "
                           f"(or __graft_entry__.build()); there is no fallback")
    L = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(status: int) -> None:
    if status != OK:
        msg = load().hgb_last_error().decode(errors="replace")
        raise HgbError(status, msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args))
