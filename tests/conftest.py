import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))

EMUL_SO = os.path.join(ROOT, "tests", "_build", "libpa_emul.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def gpu_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def build_emulator() -> str:
    """Host replay of the kernels' lane pipeline (test-only library)."""
    csrc = os.path.join(ROOT, "poy5_gb300", "csrc")
    srcs = [os.path.join(ROOT, "tests", "pa_emul.cpp"), os.path.join(csrc, "pa_tables.cpp")]
    deps = srcs + [os.path.join(csrc, f) for f in ("pa_core.cuh", "pa_tables.h", "pa_newkk.cuh",
                                                    "pa_ukk3.cuh")]
    if (not os.path.exists(EMUL_SO) or
            any(os.path.getmtime(d) > os.path.getmtime(EMUL_SO) for d in deps)):
        os.makedirs(os.path.dirname(EMUL_SO), exist_ok=True)
        subprocess.run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", csrc,
                        "-Wno-unknown-pragmas", "-o", EMUL_SO, *srcs], check=True)
    return EMUL_SO


@pytest.fixture(scope="session")
def oracle():
    from oracle_lib import Oracle
    return Oracle("port")


@pytest.fixture(scope="session")
def ctx():
    if not gpu_available():
        pytest.skip("no CUDA device")
    import poy5_gb300 as pg
    return pg.Context(0)


@pytest.fixture(scope="session")
def rng():
    return np.random.default_rng(20261203)
