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


def test_network_layer_validation_without_gpu(lib):
    """The tensor-core layer entry points check shapes, workspace size and
    alignment before any device call."""
    sz = ctypes.c_size_t(0)
    ok, bad, small = _native.LGB_OK, _native.LGB_ERR_INVALID_ARGUMENT, _native.LGB_ERR_WORKSPACE_TOO_SMALL
    assert lib.lgb_nn_conv3x3_workspace_size(4, 12, 64, 64, 32, 2, ctypes.byref(sz)) == ok
    # forward operands: im2col (4*32*32 pixels padded to 128) x (12*9 padded to 64) + weights, BF16
    assert sz.value >= (4096 * 128 + 32 * 128) * 2
    need = sz.value
    for args in [(4, 12, 64, 64, 129, 2), (4, 12, 64, 64, 32, 3), (0, 12, 64, 64, 32, 2), (4, 129, 8, 8, 32, 1)]:
        assert lib.lgb_nn_conv3x3_workspace_size(*args, ctypes.byref(sz)) == bad, args
    p = ctypes.c_void_p(1 << 20)  # never dereferenced: every check below fails before a device call
    assert lib.lgb_nn_conv3x3_forward(4, 12, 64, 64, 32, 2, 1, p, p, None, p, p, need - 1, p, None) == small
    assert lib.lgb_nn_conv3x3_forward(4, 12, 64, 64, 32, 2, 1, p, p, None, p, ctypes.c_void_p((1 << 20) + 16),
                                      need, p, None) == bad  # workspace not 256-byte aligned
    assert lib.lgb_nn_conv3x3_forward(4, 12, 64, 64, 32, 2, 1, p, p, None, p, p, need, None, None) == bad
    assert lib.lgb_nn_conv3x3_backward(4, 12, 64, 64, 32, 2, p, p, p, None, p, None, p, need - 1, p, None) == small
    assert lib.lgb_nn_linear_workspace_size(256, 2048, 512, ctypes.byref(sz)) == ok
    assert sz.value >= (512 * 2048 + 256 * 2048) * 2
    assert lib.lgb_nn_linear_workspace_size(256, 0, 512, ctypes.byref(sz)) == bad
    assert lib.lgb_nn_linear_forward(256, 2048, 512, 1, p, p, None, None, None, p, 1 << 30, p, None) == bad  # no output
    assert lib.lgb_nn_linear_backward(256, 2048, 512, p, p, p, None, p, None, p, 16, p, None) == small
