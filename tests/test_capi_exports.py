"""The C ABI library loads and exports every function include/*.h declares.
Only argument-validation paths are called (they return before touching CUDA),
so this runs on hosts without a GPU."""
import ctypes as C
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for hdr in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(hdr).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(vppgpu_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from imagecodingutils_gb300 import build
    build.build()
    return C.CDLL(build.LIB)


def test_header_declares_functions():
    assert len(declared_functions()) >= 25


def test_every_declared_symbol_is_exported(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_header():
    from imagecodingutils_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES), set(declared_functions()) - set(_lib.SIGNATURES)


def test_argument_validation_without_gpu(lib, orc):
    from imagecodingutils_gb300 import _lib
    L = _lib.load()
    assert L.vppgpu_ctx_create(0, None) == _lib.ERR_INVALID_ARG
    assert L.vppgpu_me_create(None, 0, 176, 144, 64, None) == _lib.ERR_INVALID_ARG
    assert L.vppgpu_me_destroy(None) == _lib.ERR_INVALID_ARG
    assert L.vppgpu_fwd4x4(None, None, 1, 0, 0, 28, 1) == _lib.ERR_INVALID_ARG
    assert L.vppgpu_rgb24_to_yuv420(None, 0, None, 64, 48, 0, 0, None, None, None) == _lib.ERR_INVALID_ARG
    assert L.vppgpu_status_string(_lib.ERR_PIXEL_RANGE).decode().startswith("luma")
    # the scalar quantiser helper is pure host code
    for val, pos, qp, intra in [(100, 0, 28, 1), (-77, 5, 10, 0), (255, 3, 0, 1), (-32768, 15, 51, 0)]:
        assert L.vppgpu_quantise_value(val, pos, qp, intra) == orc.quantise_value(val, pos, qp, intra)
