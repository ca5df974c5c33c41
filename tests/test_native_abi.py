"""CPU checks of the C ABI: the in-tree library loads and exports every
function declared in include/*.h; argument validation needs no GPU."""

import ctypes
import glob
import os
import re

import pytest

from leopard_em_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(lgb_\w+)\s*\(", src))
    return names


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_native.library_path()):
        from leopard_em_gb300 import build

        build.build()
    return _native.lib()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 10
    for n in sorted(names):
        assert hasattr(lib, n), f"{n} declared in include/ but not exported"


def test_problem_validation_without_gpu(lib):
    P = _native.MatchProblem
    n = ctypes.c_size_t(0)
    good = P(512, 512, 64, 1, 1, 100, 8)
    assert lib.lgb_match_supported(ctypes.byref(good)) == 1
    assert lib.lgb_match_workspace_size(ctypes.byref(good), ctypes.byref(n)) == 0 and n.value > 0
    for bad in [P(512, 511, 64, 1, 1, 100, 8), P(512, 512, 63, 1, 1, 100, 8), P(512, 512, 64, 0, 1, 100, 8),
                P(512, 512, 64, 1, 1, 100, 0), P(32, 32, 64, 1, 1, 100, 8)]:
        assert lib.lgb_match_workspace_size(ctypes.byref(bad), ctypes.byref(n)) == _native.LGB_ERR_INVALID_ARGUMENT
        assert lib.lgb_match_supported(ctypes.byref(bad)) == 0
    assert lib.lgb_match_supported(ctypes.byref(P(500, 512, 64, 1, 1, 10, 8))) == 0  # 500: no compiled FFT
    assert lib.lgb_match_init_stats(-1, None, None, None, None, None) == _native.LGB_ERR_INVALID_ARGUMENT
    assert lib.lgb_match_search(ctypes.byref(good), None, None, None, 0, 1, None, None, None, None, None, 0,
                                None) == _native.LGB_ERR_INVALID_ARGUMENT
    assert lib.lgb_status_string(2) == b"unsupported FFT size"


def test_status_maps_to_python_exceptions(lib):
    with pytest.raises(ValueError):
        _native.check(_native.LGB_ERR_INVALID_ARGUMENT, "x")
    with pytest.raises(RuntimeError):
        _native.check(_native.LGB_ERR_CUDA, "x")
    _native.check(_native.LGB_OK, "x")


def test_ctypes_signatures_match_header_arity(lib):
    """Every binding in _native has exactly the parameter count the header declares."""
    src = re.sub(r"/\*.*?\*/", "", open(os.path.join(ROOT, "include", "leopard_gb300.h")).read(), flags=re.S)
    for m in re.finditer(r"\b(lgb_\w+)\s*\(([^;]*?)\);", src, flags=re.S):
        name, params = m.group(1), m.group(2).strip()
        n = 0 if params in ("void", "") else len(params.split(","))
        assert name in _native._SIGNATURES, name
        assert len(_native._SIGNATURES[name][0]) == n, name
