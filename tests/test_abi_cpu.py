"""C-ABI library checks that need no GPU: it builds for sm_103a, loads, and
exports every entry point include/cafe_gb300.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from cafe5_gb300 import build
    build.build()
    return ctypes.CDLL(build.LIB)


def header_functions():
    text = open(os.path.join(ROOT, "include", "cafe_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cafe_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = header_functions()
    for n in ["cafe_ctx_create", "cafe_tree_upload", "cafe_families_upload", "cafe_prior_set",
              "cafe_error_model_set", "cafe_matrices_build", "cafe_matrix_get", "cafe_score", "cafe_submit",
              "cafe_poll"]:
        assert n in names


def test_library_exports_every_header_symbol(lib):
    for n in header_functions():
        assert hasattr(lib, n), n


def test_python_binding_covers_every_symbol():
    from cafe5_gb300 import _lib
    assert sorted(_lib.EXPORTS) == header_functions()


def test_status_strings_and_saturation_without_gpu(lib):
    from cafe5_gb300 import _lib
    L = _lib.load()
    assert L.cafe_status_string(0) == b"ok"
    assert L.cafe_status_string(2) == b"missing matrix"
    # matrix_cache::is_saturated: test.cpp:1639-1644
    assert L.cafe_is_saturated(25.0, 0.05) == 1
    assert L.cafe_is_saturated(25.0, 0.01) == 0
    assert L.cafe_version() >= 1


def test_context_creation_fails_cleanly_without_gpu(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from cafe5_gb300 import _lib
    L = _lib.load()
    h = ctypes.c_void_p()
    cfg = _lib.Config(0, 0, 1, 0)
    assert L.cafe_ctx_create(ctypes.byref(cfg), ctypes.byref(h)) == 7   # CAFE_ERR_CUDA, no crash
