"""Python front end of libgnlm.so (the C ABI declared in include/nlm.h).

Every call goes through ctypes into the CUDA library; there is no CPU or
framework fallback.  If the library is missing, ``lib()`` raises.  PyTorch is
used only to own device memory and streams: tensors are passed as raw device
pointers.
"""
import ctypes
import os
import subprocess

_HERE = os.path.dirname(os.path.abspath(__file__))
PKG_DIR = os.path.dirname(_HERE)
REPO_DIR = os.path.dirname(PKG_DIR)
LIB_DIR = os.path.join(PKG_DIR, "lib")
# GNLM_LIB selects another build of the library, e.g. lib/libgnlm_checked.so (the
# NLM_BOUNDS_CHECK build, whose kernels verify their index ranges at run time).
LIB_PATH = os.environ.get("GNLM_LIB") or os.path.join(LIB_DIR, "libgnlm.so")
CHECKED_LIB_PATH = os.path.join(LIB_DIR, "libgnlm_checked.so")
LEGACY_LIB_PATH = os.path.join(LIB_DIR, "libgnlm_legacy.so")
HEADER_DIR = os.path.join(REPO_DIR, "include")

NLM_OK = 0
NLM_ERR_INVALID_ARG = -1
NLM_ERR_UNSUPPORTED = -2
NLM_ERR_CUDA = -3
NLM_ERR_WORKSPACE = -4
NLM_ERR_DEVICE = -5
NLM_ERR_NO_DEVICE = -6

NLM_U8, NLM_F16, NLM_F32 = 0, 1, 2
NLM_FLAG_FP16_STORAGE = 0x1
NLM_FLAG_PREPADDED = 0x2

_lib = None


class NLMVolume(ctypes.Structure):
    """Mirror of struct nlm_volume in include/nlm.h."""
    _fields_ = [("d_in", ctypes.c_void_p), ("in_dtype", ctypes.c_int), ("X", ctypes.c_int),
                ("Y", ctypes.c_int), ("Z", ctypes.c_int), ("sr", ctypes.c_int),
                ("pr", ctypes.c_int), ("h", ctypes.c_float), ("d_out", ctypes.c_void_p),
                ("d_zsum", ctypes.c_void_p)]


class NLMError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"nlm status {code}: {msg}")
        self.code = code


def build(jobs=8, extra_nvflags=None):
    """Compile libgnlm.so (+ legacy shim and driver) for sm_103a with make."""
    cmd = ["make", "-s", "-C", PKG_DIR, f"-j{jobs}"]
    if extra_nvflags:
        cmd.append(f"EXTRA_NVFLAGS={extra_nvflags}")
    subprocess.run(cmd, check=True)


def lib():
    """Load libgnlm.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run gnlm.build() (nvcc, sm_103a)")
    L = ctypes.CDLL(LIB_PATH)
    vp, sz, i, u, f = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_uint, ctypes.c_float
    L.nlm_version.restype = ctypes.c_char_p
    L.nlm_last_error.restype = ctypes.c_char_p
    L.nlm_device_status.argtypes = [ctypes.POINTER(ctypes.c_uint)]
    L.nlm_release_cached.restype = i
    L.nlm_test_set_fault.argtypes = [u]
    L.nlm3d_workspace_bytes.argtypes = [i, i, i, i, i, u]
    L.nlm3d_workspace_bytes.restype = sz
    L.nlm3d_forward.argtypes = [vp, i, i, i, i, i, i, f, vp, vp, u, vp, sz, vp]
    L.nlm3d_forward_host.argtypes = [vp, i, i, i, i, i, i, f, vp, u]
    L.nlm3d_adjoint_workspace_bytes.argtypes = [i, i, i, i, i]
    L.nlm3d_adjoint_workspace_bytes.restype = sz
    L.nlm3d_adjoint.argtypes = [vp, vp, vp, vp, i, i, i, i, i, f, vp, vp, vp, sz, vp]
    L.nlm3d_batch_create.argtypes = [ctypes.POINTER(NLMVolume), i, u, ctypes.POINTER(vp)]
    L.nlm3d_batch_run.argtypes = [vp, vp]
    L.nlm3d_batch_autotune.argtypes = [vp, ctypes.POINTER(ctypes.c_float), vp]
    L.nlm3d_batch_set_variant.argtypes = [vp, i]
    L.nlm3d_batch_info.argtypes = [vp, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(sz)]
    L.nlm3d_batch_destroy.argtypes = [vp]
    L.nlm3d_forward_batched.argtypes = [ctypes.POINTER(NLMVolume), i, vp]
    L.nlm_variant_count.argtypes = [i, u]
    L.nlm_set_variant.argtypes = [i, i, i, u, i]
    L.nlm_get_variant.argtypes = [i, i, i, u]
    L.nlm_autotune.argtypes = [i, i, i, i, i, i, u, ctypes.POINTER(ctypes.c_float), vp]
    L.nlm3d_forward_noalloc.argtypes = [vp, i, i, i, i, i, i, f, vp, vp, u, vp]
    L.nlm3d_stage.argtypes = [vp, i, i, i, i, i, i, f, u, vp, sz, vp]
    L.nlm3d_forward_staged.argtypes = [vp, sz, i, i, i, i, i, f, vp, vp, u, vp]
    L.nlm2d_workspace_bytes.argtypes = [i, i, i, i, u]
    L.nlm2d_workspace_bytes.restype = sz
    L.nlm2d_forward.argtypes = [vp, i, i, i, i, i, f, vp, vp, u, vp, sz, vp]
    L.nlm2d_forward_host.argtypes = [vp, i, i, i, i, i, f, vp, u]
    _lib = L
    return L


def last_error():
    return lib().nlm_last_error().decode()


def check(rc):
    if rc != NLM_OK:
        raise NLMError(rc, last_error())
    return rc


def check_nonneg(rc):
    if rc < 0:
        raise NLMError(rc, last_error())
    return rc


def device_status():
    """(status, flags): reads and clears the device error word (synchronises)."""
    flags = ctypes.c_uint(0)
    rc = lib().nlm_device_status(ctypes.byref(flags))
    return rc, flags.value


# ----------------------------------------------------------------- torch glue
def _torch():
    import torch
    return torch


def _dtype_code(t):
    torch = _torch()
    return {torch.uint8: NLM_U8, torch.float16: NLM_F16, torch.float32: NLM_F32}[t.dtype]


def _stream_ptr(stream):
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def nlm3d_forward(x, sr, pr, h, fp16_storage=False, prepadded=False, return_zsum=False,
                  out=None, zsum=None, workspace=None, stream=None, shape=None):
    """3D NLM of a CUDA tensor [Z, Y, X] (uint8/float16/float32) -> float32 [Z, Y, X].

    With prepadded=True, ``x`` is the reference's padded layout and ``shape``
    gives the unpadded (Z, Y, X).
    """
    torch = _torch()
    assert x.is_cuda and x.is_contiguous()
    Z, Y, X = shape if shape is not None else x.shape
    flags = (NLM_FLAG_FP16_STORAGE if fp16_storage else 0) | (NLM_FLAG_PREPADDED if prepadded else 0)
    if out is None:
        out = torch.empty((Z, Y, X), device=x.device, dtype=torch.float32)
    if return_zsum and zsum is None:
        zsum = torch.empty((Z, Y, X), device=x.device, dtype=torch.float32)
    ws_ptr, ws_bytes = None, 0
    if workspace is not None:
        ws_ptr, ws_bytes = ctypes.c_void_p(workspace.data_ptr()), workspace.numel() * workspace.element_size()
    check(lib().nlm3d_forward(_ptr(x), _dtype_code(x), X, Y, Z, sr, pr, float(h), _ptr(out),
                              _ptr(zsum), flags, ws_ptr, ws_bytes, _stream_ptr(stream)))
    return (out, zsum) if return_zsum else out


def nlm3d_workspace_bytes(shape, sr, pr, fp16_storage=False):
    Z, Y, X = shape
    return int(lib().nlm3d_workspace_bytes(X, Y, Z, sr, pr,
                                           NLM_FLAG_FP16_STORAGE if fp16_storage else 0))


def nlm3d_stage(x, sr, pr, h, workspace, fp16_storage=False, prepadded=False, stream=None,
                shape=None):
    """Stage (pad, convert, pre-scale) ``x`` into the uint8 CUDA tensor ``workspace``."""
    Z, Y, X = shape if shape is not None else x.shape
    flags = (NLM_FLAG_FP16_STORAGE if fp16_storage else 0) | (NLM_FLAG_PREPADDED if prepadded else 0)
    check(lib().nlm3d_stage(_ptr(x), _dtype_code(x), X, Y, Z, sr, pr, float(h), flags,
                            _ptr(workspace), workspace.numel() * workspace.element_size(),
                            _stream_ptr(stream)))


def nlm3d_forward_staged(workspace, shape, sr, pr, h, out, zsum=None, fp16_storage=False,
                         stream=None):
    """Run the fused 3D kernel on a volume staged by nlm3d_stage."""
    Z, Y, X = shape
    flags = NLM_FLAG_FP16_STORAGE if fp16_storage else 0
    check(lib().nlm3d_forward_staged(_ptr(workspace), workspace.numel() * workspace.element_size(),
                                     X, Y, Z, sr, pr, float(h), _ptr(out), _ptr(zsum), flags,
                                     _stream_ptr(stream)))
    return out


def nlm3d_adjoint(x, out, zsum, gout, sr, pr, h, gin=None, hgrad=None, workspace=None,
                  stream=None):
    """dL/dv (float32 [Z, Y, X]) and dL/dh (float64 CUDA scalar) of the 3D forward."""
    torch = _torch()
    Z, Y, X = x.shape
    if gin is None:
        gin = torch.empty_like(x)
    if hgrad is None:
        hgrad = torch.zeros(1, dtype=torch.float64, device=x.device)
    ws_ptr, ws_bytes = None, 0
    if workspace is not None:
        ws_ptr, ws_bytes = ctypes.c_void_p(workspace.data_ptr()), workspace.numel() * workspace.element_size()
    check(lib().nlm3d_adjoint(_ptr(x), _ptr(out), _ptr(zsum), _ptr(gout), X, Y, Z, sr, pr,
                              float(h), _ptr(gin), _ptr(hgrad), ws_ptr, ws_bytes,
                              _stream_ptr(stream)))
    return gin, hgrad


def nlm3d_forward_batched(volumes, stream=None):
    """One-shot batched forward (plan built, run once and freed; synchronous).

    ``volumes`` is a list of (tensor [Z, Y, X], sr, pr, h); returns the outputs."""
    torch = _torch()
    inputs = [v[0].contiguous() for v in volumes]
    outputs = [torch.empty(t.shape, dtype=torch.float32, device=t.device) for t in inputs]
    arr = (NLMVolume * len(volumes))()
    for k, ((_, sr, pr, h), x, o) in enumerate(zip(volumes, inputs, outputs)):
        Z, Y, X = x.shape
        arr[k] = NLMVolume(x.data_ptr(), _dtype_code(x), X, Y, Z, sr, pr, float(h), o.data_ptr(),
                           None)
    check(lib().nlm3d_forward_batched(arr, len(volumes), _stream_ptr(stream)))
    return outputs


class BatchPlan:
    """A batched 3D plan over CUDA tensors (one persistent, graph-captured launch).

    ``volumes`` is a list of (tensor [Z, Y, X], sr, pr, h); outputs are allocated here.
    """

    N_VARIANTS = 4

    def __init__(self, volumes, with_zsum=False):
        torch = _torch()
        self.inputs = [v[0].contiguous() for v in volumes]
        self.outputs = [torch.empty(t.shape, dtype=torch.float32, device=t.device)
                        for t in self.inputs]
        self.zsums = [torch.empty_like(o) for o in self.outputs] if with_zsum else None
        arr = (NLMVolume * len(volumes))()
        for k, ((t, sr, pr, h), x, o) in enumerate(zip(volumes, self.inputs, self.outputs)):
            Z, Y, X = x.shape
            arr[k] = NLMVolume(x.data_ptr(), _dtype_code(x), X, Y, Z, sr, pr, float(h),
                               o.data_ptr(), self.zsums[k].data_ptr() if with_zsum else None)
        self._arr = arr
        self.handle = ctypes.c_void_p()
        check(lib().nlm3d_batch_create(arr, len(volumes), 0, ctypes.byref(self.handle)))

    def run(self, stream=None):
        check(lib().nlm3d_batch_run(self.handle, _stream_ptr(stream)))
        return self.outputs

    def autotune(self, stream=None):
        times = (ctypes.c_float * self.N_VARIANTS)()
        best = check_nonneg(lib().nlm3d_batch_autotune(self.handle, times, _stream_ptr(stream)))
        return best, list(times)

    def set_variant(self, v):
        check(lib().nlm3d_batch_set_variant(self.handle, int(v)))

    def info(self):
        n, v, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t()
        check(lib().nlm3d_batch_info(self.handle, ctypes.byref(n), ctypes.byref(v), ctypes.byref(b)))
        return {"items": n.value, "variant": v.value, "device_bytes": b.value}

    def close(self):
        if self.handle:
            lib().nlm3d_batch_destroy(self.handle)
            self.handle = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def variant_count(dims, fp16_storage=False):
    return check_nonneg(lib().nlm_variant_count(dims, NLM_FLAG_FP16_STORAGE if fp16_storage else 0))


def set_variant(dims, sr, pr, variant, fp16_storage=False):
    check(lib().nlm_set_variant(dims, sr, pr, NLM_FLAG_FP16_STORAGE if fp16_storage else 0,
                                int(variant)))


def get_variant(dims, sr, pr, fp16_storage=False):
    return check_nonneg(lib().nlm_get_variant(dims, sr, pr,
                                              NLM_FLAG_FP16_STORAGE if fp16_storage else 0))


def autotune(dims, shape, sr, pr, fp16_storage=False, stream=None):
    """Time every tile-shape variant; returns (best_index, times_ms list)."""
    flags = NLM_FLAG_FP16_STORAGE if fp16_storage else 0
    n = variant_count(dims, fp16_storage)
    times = (ctypes.c_float * n)()
    Z, Y, X = shape if len(shape) == 3 else (1,) + tuple(shape)
    best = check_nonneg(lib().nlm_autotune(dims, X, Y, Z, sr, pr, flags, times, _stream_ptr(stream)))
    return best, list(times)


def nlm2d_forward(x, sr, pr, h, fp16_storage=False, prepadded=False, return_zsum=False,
                  out=None, zsum=None, workspace=None, stream=None, shape=None):
    """2D NLM of a CUDA tensor [Y, X] -> float32 [Y, X]."""
    torch = _torch()
    assert x.is_cuda and x.is_contiguous()
    Y, X = shape if shape is not None else x.shape
    flags = (NLM_FLAG_FP16_STORAGE if fp16_storage else 0) | (NLM_FLAG_PREPADDED if prepadded else 0)
    if out is None:
        out = torch.empty((Y, X), device=x.device, dtype=torch.float32)
    if return_zsum and zsum is None:
        zsum = torch.empty((Y, X), device=x.device, dtype=torch.float32)
    ws_ptr, ws_bytes = None, 0
    if workspace is not None:
        ws_ptr, ws_bytes = ctypes.c_void_p(workspace.data_ptr()), workspace.numel() * workspace.element_size()
    check(lib().nlm2d_forward(_ptr(x), _dtype_code(x), X, Y, sr, pr, float(h), _ptr(out),
                              _ptr(zsum), flags, ws_ptr, ws_bytes, _stream_ptr(stream)))
    return (out, zsum) if return_zsum else out


def _np_dtype_code(a):
    import numpy as np
    return {np.dtype(np.uint8): NLM_U8, np.dtype(np.float16): NLM_F16,
            np.dtype(np.float32): NLM_F32}[a.dtype]


def nlm3d_forward_host(a, sr, pr, h, fp16_storage=False, prepadded=False, shape=None, out=None):
    """Host-buffer 3D form (numpy in, numpy out; synchronous)."""
    import numpy as np
    a = np.ascontiguousarray(a)
    Z, Y, X = shape if shape is not None else a.shape
    flags = (NLM_FLAG_FP16_STORAGE if fp16_storage else 0) | (NLM_FLAG_PREPADDED if prepadded else 0)
    if out is None:
        out = np.empty((Z, Y, X), np.float32)
    check(lib().nlm3d_forward_host(a.ctypes.data_as(ctypes.c_void_p), _np_dtype_code(a), X, Y, Z,
                                   sr, pr, float(h), out.ctypes.data_as(ctypes.c_void_p), flags))
    return out


def nlm2d_forward_host(a, sr, pr, h, fp16_storage=False, prepadded=False, shape=None, out=None):
    """Host-buffer 2D form (numpy in, numpy out; synchronous)."""
    import numpy as np
    a = np.ascontiguousarray(a)
    Y, X = shape if shape is not None else a.shape
    flags = (NLM_FLAG_FP16_STORAGE if fp16_storage else 0) | (NLM_FLAG_PREPADDED if prepadded else 0)
    if out is None:
        out = np.empty((Y, X), np.float32)
    check(lib().nlm2d_forward_host(a.ctypes.data_as(ctypes.c_void_p), _np_dtype_code(a), X, Y, sr,
                                   pr, float(h), out.ctypes.data_as(ctypes.c_void_p), flags))
    return out
