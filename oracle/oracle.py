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
        _ip = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
        L.oracle_nlm3d_blocks_sep_f32.argtypes = [_f32p, _i, _i, _i, _i, _i, ctypes.c_float,
                                                  _i, _ip, _i, _i, _i, _f32p]
        L.oracle_nlm3d_blocks_sep_f64.argtypes = [_f64p, _i, _i, _i, _i, _i, ctypes.c_double,
                                                  _i, _ip, _i, _i, _i, _f64p]
        L.oracle_nlm3d_fd_grad_f64.argtypes = [_f64p, _i, _i, _i, _i, _i, ctypes.c_double,
                                               _f64p, _i, _ip, ctypes.c_double, _f64p]
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


def nlm3d_blocks(v, sr, pr, h, origins, size, dtype=np.float64):
    """Separable-form NLM of several boxes of a full volume: origins is a list of
    (z0, y0, x0), size = (nz, ny, nx); returns an array [len(origins), nz, ny, nx]."""
    v = np.ascontiguousarray(v, dtype=dtype)
    Z, Y, X = v.shape
    nz, ny, nx = size
    org = np.ascontiguousarray([[x0, y0, z0] for (z0, y0, x0) in origins], dtype=np.int32)
    out = np.empty((len(origins), nz, ny, nx), dtype)
    fn = lib().oracle_nlm3d_blocks_sep_f32 if dtype == np.float32 else \
        lib().oracle_nlm3d_blocks_sep_f64
    fn(v, X, Y, Z, sr, pr, h, len(origins), org.ravel(), nx, ny, nz, out)
    return out


def border_blocks(shape, size):
    """Origins (z0, y0, x0) of boxes of `size` at the 8 corners, the 6 face centres
    and the centre of a volume: every border face and edge is sampled."""
    out = []
    lo_hi = [(0, (n - s) // 2, n - s) for n, s in zip(shape, size)]
    for kz, ky, kx in [(a, b, c) for a in (0, 2) for b in (0, 2) for c in (0, 2)] + \
            [(0, 1, 1), (2, 1, 1), (1, 0, 1), (1, 2, 1), (1, 1, 0), (1, 1, 2), (1, 1, 1)]:
        out.append((lo_hi[0][kz], lo_hi[1][ky], lo_hi[2][kx]))
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


def fd_voxel_grad(v, sr, pr, h, g, voxels, eps=1e-5):
    """FP64 central differences of L = sum(g * nlm3d(v)) with respect to the voxels
    (list of (z, y, x)); only the outputs within sr + pr of a voxel are re-evaluated."""
    v = np.ascontiguousarray(v, dtype=np.float64)
    g = np.ascontiguousarray(g, dtype=np.float64)
    Z, Y, X = v.shape
    idx = np.ascontiguousarray([[x, y, z] for (z, y, x) in voxels], dtype=np.int32)
    fd = np.empty(len(voxels))
    lib().oracle_nlm3d_fd_grad_f64(v, X, Y, Z, sr, pr, h, g, len(voxels), idx.ravel(), eps, fd)
    return fd


def fd_sample_voxels(shape, n, seed):
    """n distinct voxels (z, y, x): the 8 corners and one voxel on each face, the rest
    uniform at random (seeded)."""
    rng = np.random.default_rng(seed)
    Z, Y, X = shape
    vox = [(z, y, x) for z in (0, Z - 1) for y in (0, Y - 1) for x in (0, X - 1)]
    vox += [(0, Y // 2, X // 3), (Z - 1, Y // 3, X // 2), (Z // 2, 0, X // 4),
            (Z // 3, Y - 1, X // 2), (Z // 4, Y // 2, 0), (Z // 2, Y // 4, X - 1)]
    seen = set(vox)
    while len(vox) < n:
        c = tuple(int(rng.integers(0, s)) for s in shape)
        if c not in seen:
            seen.add(c)
            vox.append(c)
    return vox


def fd_h_grad(v, sr, pr, h, g, eps=1e-6):
    """FP64 central difference of L = sum(g * nlm3d(v)) with respect to h, from two
    full-volume FP64 separable forwards."""
    g = np.asarray(g, dtype=np.float64)
    lp = float((nlm3d(v, sr, pr, h + eps, dtype=np.float64) * g).sum())
    lm = float((nlm3d(v, sr, pr, h - eps, dtype=np.float64) * g).sum())
    return (lp - lm) / (2 * eps)


def pad_reflect101(v, H):
    """REFLECT_101 padding by H on every axis (numpy, any H)."""
    idx = []
    for n in v.shape:
        idx.append(np.array([reflect101(i - H, n) for i in range(n + 2 * H)]))
    return v[np.ix_(*idx)]
