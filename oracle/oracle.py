"""ctypes front end of the NLM oracle (oracle/nlm_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and
by bench.py's CPU-baseline leg, always as the checker or the timed CPU
baseline, never as the product path.  The product is the CUDA library behind
include/nlm.h and has no CPU fallback.

The arithmetic follows the reference's generic kernels (3DNLM/main.cu:28-238 and
2D NLM/11x11/main.cu:383-468); see nlm_oracle.c for the line-by-line mapping.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")
_i = ctypes.c_int

FORM_DIRECT = 0
FORM_SEPARABLE = 1


def build():
    """Compile liboracle.so with the committed Makefile (portable C, OpenMP)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        vp = ctypes.c_void_p
        L.oracle_reflect101.argtypes = [ctypes.c_long, ctypes.c_long]
        L.oracle_reflect101.restype = ctypes.c_long
        L.oracle_set_threads.argtypes = [_i]
        L.oracle_max_threads.restype = _i
        L.oracle_nlm3d_f32.argtypes = [_f32p, _i, _i, _i, _i, _i, ctypes.c_float, _f32p, vp, _i]
        L.oracle_nlm3d_f64.argtypes = [_f64p, _i, _i, _i, _i, _i, ctypes.c_double, _f64p, vp, _i]
        L.oracle_nlm2d_f32.argtypes = [_f32p, _i, _i, _i, _i, ctypes.c_float, _f32p, vp, _i]
        L.oracle_nlm2d_f64.argtypes = [_f64p, _i, _i, _i, _i, ctypes.c_double, _f64p, vp, _i]
        L.oracle_nlm3d_padded_u8.argtypes = [_u8p, _i, _i, _i, _i, _i, ctypes.c_float, _f32p, _i]
        L.oracle_nlm2d_padded_u8.argtypes = [_u8p, _i, _i, _i, _i, ctypes.c_float, _f32p, _i]
        L.oracle_nlm3d_region_f32.argtypes = [_f32p, _i, _i, _i, _i, _i, ctypes.c_float,
                                              _i, _i, _i, _i, _i, _i, _f32p]
        L.oracle_nlm3d_region_f64.argtypes = [_f64p, _i, _i, _i, _i, _i, ctypes.c_double,
                                              _i, _i, _i, _i, _i, _i, _f64p]
        L.oracle_nlm3d_adjoint_f64.argtypes = [_f64p, _i, _i, _i, _i, _i, ctypes.c_double,
                                               _f64p, _f64p, ctypes.POINTER(ctypes.c_double), vp]
        _lib = L
    return _lib


def _zs_ptr(z):
    return None if z is None else z.ctypes.data_as(ctypes.c_void_p)


def set_threads(n):
    lib().oracle_set_threads(int(n))


def max_threads():
    return int(lib().oracle_max_threads())


def reflect101(i, n):
    return int(lib().oracle_reflect101(int(i), int(n)))


def nlm3d(v, sr, pr, h, form=FORM_SEPARABLE, dtype=np.float32, return_z=False):
    """3D NLM of a [Z][Y][X] volume with REFLECT_101 borders on every axis."""
    v = np.ascontiguousarray(v, dtype=dtype)
    Z, Y, X = v.shape
    out = np.empty_like(v)
    zs = np.empty_like(v) if return_z else None
    fn = lib().oracle_nlm3d_f32 if dtype == np.float32 else lib().oracle_nlm3d_f64
    fn(v, X, Y, Z, sr, pr, h, out, _zs_ptr(zs), form)
    return (out, zs) if return_z else out


def nlm3d_region(v, sr, pr, h, origin, size, dtype=np.float64):
    """Direct-form NLM of the box origin=(z0, y0, x0), size=(nz, ny, nx) of a full volume."""
    v = np.ascontiguousarray(v, dtype=dtype)
    Z, Y, X = v.shape
    z0, y0, x0 = origin
    nz, ny, nx = size
    out = np.empty((nz, ny, nx), dtype)
    fn = lib().oracle_nlm3d_region_f32 if dtype == np.float32 else lib().oracle_nlm3d_region_f64
    fn(v, X, Y, Z, sr, pr, h, x0, y0, z0, nx, ny, nz, out)
    return out


def nlm2d(v, sr, pr, h, form=FORM_SEPARABLE, dtype=np.float32, return_z=False):
    """2D NLM of a [Y][X] image with REFLECT_101 borders."""
    v = np.ascontiguousarray(v, dtype=dtype)
    Y, X = v.shape
    out = np.empty_like(v)
    zs = np.empty_like(v) if return_z else None
    fn = lib().oracle_nlm2d_f32 if dtype == np.float32 else lib().oracle_nlm2d_f64
    fn(v, X, Y, sr, pr, h, out, _zs_ptr(zs), form)
    return (out, zs) if return_z else out


def nlm3d_padded_u8(padded, X, Y, Z, SS, NS, h, form=FORM_SEPARABLE):
    """Legacy layout of the reference's NL_Means (3DNLM/main.h:6): pre-padded uchar."""
    padded = np.ascontiguousarray(padded, dtype=np.uint8)
    out = np.empty((Z, Y, X), np.float32)
    lib().oracle_nlm3d_padded_u8(padded.ravel(), X, Y, Z, SS, NS, h, out, form)
    return out


def nlm2d_padded_u8(padded, X, Y, sr_size, nb_size, h, form=FORM_SEPARABLE):
    """Legacy 2D layout (2D NLM/11x11/main.h:6): pre-padded uchar image."""
    padded = np.ascontiguousarray(padded, dtype=np.uint8)
    out = np.empty((Y, X), np.float32)
    lib().oracle_nlm2d_padded_u8(padded.ravel(), X, Y, sr_size, nb_size, h, out, form)
    return out


def nlm3d_adjoint(v, sr, pr, h, g):
    """FP64 gradients (dL/dv, dL/dh, out) for upstream gradient g; direct form."""
    v = np.ascontiguousarray(v, dtype=np.float64)
    g = np.ascontiguousarray(g, dtype=np.float64)
    Z, Y, X = v.shape
    gin = np.empty_like(v)
    out = np.empty_like(v)
    gh = ctypes.c_double(0.0)
    lib().oracle_nlm3d_adjoint_f64(v, X, Y, Z, sr, pr, h, g, gin, ctypes.byref(gh),
                                   out.ctypes.data_as(ctypes.c_void_p))
    return gin, gh.value, out


def pad_reflect101(v, H):
    """REFLECT_101 padding by H on every axis (numpy, any H)."""
    idx = []
    for n in v.shape:
        idx.append(np.array([reflect101(i - H, n) for i in range(n + 2 * H)]))
    return v[np.ix_(*idx)]
