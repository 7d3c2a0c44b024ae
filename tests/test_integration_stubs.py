"""The POY-side stub library (integration/poy_stubs.c) compiles against POY's
own headers (seq.h, cm.h) and include/poyalgn.h with the caml header shim
the oracle build uses, defines every external it replaces (with the bytecode
twins), and links against libpoyalgn.so with no undefined symbol left.
Skipped where the POY sources are absent."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from build_oracle import DEFAULT_REF_SRC  # noqa: E402

STUBS = os.path.join(ROOT, "integration", "poy_stubs.c")
LIBDIR = os.path.join(ROOT, "poy5_gb300")

# every external of the path (src/algn.c, src/seq.c, src/newkkonen.c,
# src/ukkCommon.c) the stub library replaces, bytecode twins included
EXTERNALS = [
    "algn_CAML_simple_2", "algn_CAML_backtrace_2d", "algn_CAML_backtrace_2d_bc",
    "algn_CAML_align_2d", "algn_CAML_align_2d_bc", "algn_CAML_limit_2",
    "algn_CAML_limit_2_bc", "algn_CAML_backtrace_2d_limit",
    "algn_CAML_backtrace_2d_limit_bc", "algn_CAML_align_affine_3",
    "algn_CAML_align_affine_3_bc", "algn_CAML_cost_affine_3", "algn_CAML_ancestor_2",
    "algn_CAML_worst_2", "algn_CAML_verify_2", "seq_CAML_median_2_no_gaps",
    "seq_CAML_median_2_with_gaps", "newkkonen_CAML_algn_affine",
    "newkkonen_CAML_backtrace_affine", "newkkonen_CAML_backtrace_affine_bc",
    "newkkonen_CAML_get_k", "powell_3D_align", "powell_3D_align_bc",
]

needs_poy = pytest.mark.skipif(not os.path.isfile(os.path.join(DEFAULT_REF_SRC, "seq.h")),
                               reason="POY sources absent")


def _cc(*args):
    subprocess.run(["gcc", "-std=gnu11", "-fgnu89-inline", "-fPIC", "-Werror", "-Wall",
                    "-Wno-unused-variable", "-I", os.path.join(ROOT, "oracle", "shim"),
                    "-I", DEFAULT_REF_SRC, "-I", os.path.join(ROOT, "include"), *args],
                   check=True)


def _symbols(path, *flags):
    out = subprocess.run(["nm", *flags, path], check=True, capture_output=True,
                         text=True).stdout
    return {line.split()[-1] for line in out.splitlines() if line.strip()}


@needs_poy
def test_integration_stubs_compile_and_link(tmp_path):
    obj = str(tmp_path / "poy_stubs.o")
    _cc("-O2", "-c", STUBS, "-o", obj)
    defined = _symbols(obj, "--defined-only")
    missing = [s for s in EXTERNALS if s not in defined]
    assert not missing, missing
    # every libpoyalgn entry point the stubs call is exported by the library
    lib = os.path.join(LIBDIR, "libpoyalgn.so")
    if not os.path.exists(lib):
        pytest.skip("libpoyalgn.so not built")
    exported = _symbols(lib, "-D", "--defined-only")
    undefined = _symbols(obj, "-u")
    calls = sorted(s for s in undefined if s.startswith("poyalgn_"))
    assert len(calls) >= 15, calls
    assert not [s for s in calls if s not in exported]
    # and the stub library links with nothing left undefined
    rt = str(tmp_path / "stub_runtime.o")
    _cc("-O2", "-c", os.path.join(ROOT, "tests", "stub_runtime.c"), "-o", rt)
    so = str(tmp_path / "libpoystubs.so")
    subprocess.run(["gcc", "-shared", "-o", so, obj, rt, "-L", LIBDIR, "-lpoyalgn",
                    "-Wl,--no-undefined", "-Wl,-rpath," + LIBDIR], check=True)
    needed = subprocess.run(["readelf", "-d", so], check=True, capture_output=True,
                            text=True).stdout
    assert "libpoyalgn.so" in needed
