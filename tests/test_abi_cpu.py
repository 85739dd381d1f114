"""CPU tests of the C ABI: the library loads, exports every entry point the
headers in include/ declare, and rejects bad arguments on the host (no GPU
work is issued by any of these calls)."""
import ctypes
import os
import re

import pytest

import gnlm


def _declared_functions(header):
    text = open(header).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    names = re.findall(r"\b(nlm[a-z0-9_]*)\s*\([^;{]*\)\s*;", text)
    return sorted(set(names))


@pytest.fixture(scope="module")
def L(gnlm_lib):
    return gnlm_lib.lib()


def test_headers_declare_entry_points():
    names = _declared_functions(os.path.join(gnlm.HEADER_DIR, "nlm.h"))
    for must in ("nlm3d_forward", "nlm2d_forward", "nlm_last_error", "nlm3d_forward_host"):
        assert must in names


def test_library_exports_every_declared_symbol(L):
    for hdr in sorted(os.listdir(gnlm.HEADER_DIR)):
        if not hdr.endswith(".h"):
            continue
        for name in _declared_functions(os.path.join(gnlm.HEADER_DIR, hdr)):
            assert hasattr(L, name), f"{name} declared in {hdr} but not exported"


def test_legacy_shim_exports_reference_signatures(gnlm_lib):
    legacy = ctypes.CDLL(gnlm_lib.LEGACY_LIB_PATH)
    # NLMeansProcessor::NL_Means(unsigned char*, float*) and the 2D overload
    assert hasattr(legacy, "_ZN16NLMeansProcessor8NL_MeansEPhPf")
    assert hasattr(legacy, "_ZN16NLMeansProcessor8NL_MeansEPhPfiiiiii")


def test_noalloc_checks_arguments_before_its_size_limit(L):
    """A bad pointer, dtype, h or flag on a volume too large for the allocation-free
    entry point's array is reported as the bad argument, not as a size problem (the
    checks run on the host; no device work is issued)."""
    P = ctypes.c_void_p
    big = (400, 400, 400)
    assert L.nlm3d_workspace_bytes(*big, 3, 1, 0) > 16 << 20
    one = P(256)  # never dereferenced: every call below fails its host checks first
    calls = [(None, gnlm.NLM_F32, 0.05, 0), (one, 7, 0.05, 0), (one, gnlm.NLM_F32, -1.0, 0),
             (one, gnlm.NLM_F32, 0.05, 0x80)]
    for d_in, dt, h, flags in calls:
        rc = L.nlm3d_forward_noalloc(d_in, dt, *big, 3, 1, h, one, None, flags, None)
        assert rc == gnlm.NLM_ERR_INVALID_ARG, (d_in, dt, h, flags, gnlm.last_error())
    rc = L.nlm3d_forward_noalloc(one, gnlm.NLM_F32, *big, 9, 1, 0.05, one, None, 0, None)
    assert rc == gnlm.NLM_ERR_UNSUPPORTED


def test_fault_hook_is_inert_in_the_production_build(L):
    """nlm_test_set_fault exists only to drive the bounded waits of the checked test
    build; the production library refuses it before touching any device."""
    assert L.nlm_test_set_fault(1) == gnlm.NLM_ERR_UNSUPPORTED
    assert "test build" in gnlm.last_error()


def test_version(L):
    assert b"sm_103a" in L.nlm_version()


def test_workspace_query_is_pure_host(L):
    b32 = L.nlm3d_workspace_bytes(64, 64, 64, 3, 1, 0)
    b16 = L.nlm3d_workspace_bytes(64, 64, 64, 3, 1, gnlm.NLM_FLAG_FP16_STORAGE)
    # padded 72^3, x stride rounded to 16 bytes, 256-byte aligned
    assert b32 == ((72 * 72 * 72 * 4 + 255) // 256) * 256
    # FP16 storage: two row-pair copies (37 pairs of 72 padded rows) of half2
    assert b16 == 2 * (((72 * 37 * 72 * 4) + 255) // 256) * 256
    assert L.nlm3d_workspace_bytes(0, 64, 64, 3, 1, 0) == 0
    assert L.nlm2d_workspace_bytes(2048, 2048, 5, 2, 0) == ((2064 * 2062 * 4 + 255) // 256) * 256
    # large patch (search 13, patch 17 on 512 x 512 x 16): staged volume padded by 14
    # (x stride rounded to 4 floats), then four buffers of one (Z, num) float pair per
    # voxel (each tile's passes may be split between two CTAs, and from search radius 3
    # each pass's x offsets are split between two more); search radius 2 keeps two
    staged = ((540 * 540 * 44 * 4 + 255) // 256) * 256
    assert L.nlm3d_workspace_bytes(512, 512, 16, 6, 8, 0) == staged + 4 * 512 * 512 * 16 * 8
    staged2 = ((532 * 532 * 36 * 4 + 255) // 256) * 256  # padded by 10, x stride 532
    assert L.nlm3d_workspace_bytes(512, 512, 16, 2, 8, 0) == staged2 + 2 * 512 * 512 * 16 * 8


@pytest.mark.parametrize("args,code", [
    # null input
    ((None, gnlm.NLM_F32, 8, 8, 8, 3, 1, 0.05, 1, None, 0, None, 0, None), gnlm.NLM_ERR_INVALID_ARG),
    # null output
    ((1, gnlm.NLM_F32, 8, 8, 8, 3, 1, 0.05, None, None, 0, None, 0, None), gnlm.NLM_ERR_INVALID_ARG),
    # bad dtype
    ((1, 7, 8, 8, 8, 3, 1, 0.05, 1, None, 0, None, 0, None), gnlm.NLM_ERR_INVALID_ARG),
    # h <= 0
    ((1, gnlm.NLM_F32, 8, 8, 8, 3, 1, 0.0, 1, None, 0, None, 0, None), gnlm.NLM_ERR_INVALID_ARG),
    # NaN h
    ((1, gnlm.NLM_F32, 8, 8, 8, 3, 1, float("nan"), 1, None, 0, None, 0, None), gnlm.NLM_ERR_INVALID_ARG),
    # negative radius
    ((1, gnlm.NLM_F32, 8, 8, 8, -1, 1, 0.05, 1, None, 0, None, 0, None), gnlm.NLM_ERR_INVALID_ARG),
    # zero extent
    ((1, gnlm.NLM_F32, 0, 8, 8, 3, 1, 0.05, 1, None, 0, None, 0, None), gnlm.NLM_ERR_INVALID_ARG),
    # unknown flag
    ((1, gnlm.NLM_F32, 8, 8, 8, 3, 1, 0.05, 1, None, 0x80, None, 0, None), gnlm.NLM_ERR_INVALID_ARG),
    # too many planes for the staging grid
    ((1, gnlm.NLM_F32, 8, 8, 70000, 3, 1, 0.05, 1, None, 0, None, 0, None), gnlm.NLM_ERR_INVALID_ARG),
    # radius combination not compiled in
    ((1, gnlm.NLM_F32, 8, 8, 8, 9, 4, 0.05, 1, None, 0, None, 0, None), gnlm.NLM_ERR_UNSUPPORTED),
    # caller workspace too small
    ((1, gnlm.NLM_F32, 8, 8, 8, 3, 1, 0.05, 1, None, 0, 256, 16, None), gnlm.NLM_ERR_WORKSPACE),
])
def test_forward_rejects_bad_arguments(L, args, code):
    args = [ctypes.c_void_p(a) if isinstance(a, int) and i in (0, 8, 11) else a
            for i, a in enumerate(args)]
    rc = L.nlm3d_forward(*args)
    assert rc == code, gnlm.last_error()
    assert gnlm.last_error() != ""


def test_last_error_is_per_thread(L):
    import threading
    L.nlm3d_forward(None, 2, 8, 8, 8, 3, 1, 0.05, None, None, 0, None, 0, None)
    main_msg = gnlm.last_error()
    seen = {}

    def worker():
        seen["msg"] = gnlm.last_error()

    t = threading.Thread(target=worker)
    t.start()
    t.join()
    assert main_msg and seen["msg"] == ""


def test_2d_rejects_bad_arguments(L):
    rc = L.nlm2d_forward(None, gnlm.NLM_F32, 8, 8, 5, 2, 0.08, None, None, 0, None, 0, None)
    assert rc == gnlm.NLM_ERR_INVALID_ARG
    rc = L.nlm2d_forward(ctypes.c_void_p(1), gnlm.NLM_F32, 8, 8, 4, 4, 0.08, ctypes.c_void_p(1),
                         None, 0, None, 0, None)
    assert rc == gnlm.NLM_ERR_UNSUPPORTED


def test_default_variants_without_autotune(L):
    """Before any autotuning the forward uses the measured per-configuration default
    (no GPU needed to read it)."""
    fp16 = gnlm.NLM_FLAG_FP16_STORAGE
    assert L.nlm_get_variant(3, 3, 1, 0) == 4   # 3D FP32 patch 3: z offsets in groups of four, 4 x 6
    assert L.nlm_get_variant(3, 5, 2, 0) == 5
    assert L.nlm_get_variant(3, 3, 2, 0) == 0
    assert L.nlm_get_variant(3, 3, 1, fp16) == 0
    assert L.nlm_get_variant(3, 6, 8, 0) == 0   # large-patch kernel, 64-plane chunks
    assert L.nlm_get_variant(2, 5, 2, 0) == 5   # 2D: two columns per lane
    assert L.nlm_get_variant(2, 10, 5, 0) == 5
    assert L.nlm_get_variant(2, 5, 2, fp16) == 0
    for dims, flags in [(3, 0), (3, fp16), (2, 0)]:
        assert L.nlm_variant_count(dims, flags) > L.nlm_get_variant(dims, 3, 1, flags)
