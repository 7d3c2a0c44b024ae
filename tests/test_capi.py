"""The C-ABI library builds, loads and exports what include/poyalgn.h declares.

No compute call is made here (no GPU on this machine); the GPU tests call
through the same entry points.
"""
import ctypes as C

import pytest


@pytest.fixture(scope="module")
def lib():
    from poy5_gb300 import build
    build.build()
    from poy5_gb300 import _lib
    return _lib.load()


def test_exports_every_declared_symbol(lib):
    from poy5_gb300 import _lib
    declared = _lib.header_symbols()
    assert len(declared) >= 15
    for name in declared:
        assert hasattr(lib, name), name


def test_build_recipe_targets_sm_103a():
    from poy5_gb300 import build
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_version_and_error_without_device(lib):
    assert lib.poyalgn_version().startswith(b"poyalgn")
    h = C.c_void_p()
    # on a machine without a GPU, init must fail loudly (no CPU fallback)
    import conftest
    if not conftest.gpu_available():
        assert lib.poyalgn_init(0, C.byref(h)) != 0
        assert lib.poyalgn_last_error()


def test_python_layer_fails_loudly_without_gpu():
    import conftest
    if conftest.gpu_available():
        pytest.skip("GPU present")
    import poy5_gb300 as pg
    with pytest.raises(pg.PoyAlgnError):
        pg.Context(0)


def test_candidate_ladders_are_valid():
    from poy5_gb300 import tune
    for affine in (False, True):
        cands = tune.candidate_ladders(affine)
        assert cands[0] == tune.default_ladder(affine)
        assert all(tune.ladder_valid(P, R, affine) for P, R in cands)
    n = tune.NCLASS
    assert not tune.ladder_valid([4] * (n - 1) + [3], [2] * n, True)
    assert not tune.ladder_valid([512] + [4] * (n - 1), [4] * n, True)   # capacity drops
    assert not tune.ladder_valid([4] * n, [8] * n, True)                 # affine R <= 4
    assert tune.ladder_valid([4] * n, [3] * n, True)                     # R = 3: affine only
    assert not tune.ladder_valid([4] * n, [3] * n, False)
    assert not tune.ladder_valid([4] * 10, [2] * 10, True)               # one per class
