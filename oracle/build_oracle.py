"""Build recipe for the oracle (test infrastructure only).

* ``oracle/libpoyoracle.so`` — the C restatement of the reference path
  (``poy_oracle.c`` + ``poy_tables.c``). Built on every machine; it is the
  checker the GPU tests, ``smoke()`` and the CPU baseline use.
* ``oracle/_ref/libpoyref.so`` (+ ``libpoyref_long.so`` with
  ``USE_LONG_SEQUENCES``) — the reference POY ``src/algn.c`` unit and
  ``src/newkkonen.c`` (+ its queue) compiled
  unmodified from the POY source tree, plus ``ref_harness.c`` and the caml
  header shim. Built only where the POY sources are present; it validates the
  restatement and generates the golden fixtures.

Run: ``python oracle/build_oracle.py [--ref-src DIR]``.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# where the POY 5.1.1 sources are (POY_REF_SRC, or --ref-src): this recipe
# compiles the reference unit from them in place; without them only the port
# is built
DEFAULT_REF_SRC = os.environ.get("POY_REF_SRC", "/root/reference/src")


def _run(cmd):
    subprocess.run(cmd, check=True)


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_port(force: bool = False) -> str:
    out = os.path.join(HERE, "libpoyoracle.so")
    srcs = [os.path.join(HERE, f) for f in ("poy_oracle.c", "poy_tables.c", "poy_ukk3.c")]
    hdrs = [os.path.join(HERE, f) for f in ("poy_oracle.h", "poy_tables.h")]
    if force or _stale(out, srcs + hdrs):
        _run(["gcc", "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp",
              "-Wall", "-Wno-unused-function", "-o", out, *srcs])
    return out


def build_ref(ref_src: str = DEFAULT_REF_SRC, force: bool = False):
    """Compile the reference algn.c unit (returns [] when sources are absent)."""
    if not os.path.isfile(os.path.join(ref_src, "algn.c")):
        return []
    outdir = os.path.join(HERE, "_ref")
    os.makedirs(outdir, exist_ok=True)
    # newkkonen.c (Algn_Newkk) and its queue; algn.c and newkkonen.c both
    # define the tentative global `backtrace_mode`, hence -fcommon.
    # ukkCommon.c + ukk.checkp.c: Powell's three-sequence alignment
    srcs = [os.path.join(ref_src, f) for f in ("algn.c", "avl.c", "zarr.c",
                                               "newkkonen.c",
                                               "queue_with_linkedlist.c",
                                               "ukkCommon.c", "ukk.checkp.c")]
    mine = [os.path.join(HERE, f) for f in ("ref_harness.c", "poy_tables.c")]
    built = []
    for name, extra in (("libpoyref.so", []),
                        ("libpoyref_long.so", ["-DUSE_LONG_SEQUENCES"])):
        out = os.path.join(outdir, name)
        if force or _stale(out, mine + [os.path.join(HERE, "shim", "caml",
                                                      "poy_caml_shim.h")]):
            # -Bsymbolic: the reference's own functions bind inside the
            # library (glibc exports a legacy `step` that ukk.checkp.c's
            # calls would otherwise reach when the library is dlopen'ed)
            _run(["gcc", "-O2", "-fgnu89-inline", "-fcommon", "-fPIC", "-shared", "-w",
                  "-Wl,-Bsymbolic",
                  *extra, "-I", os.path.join(HERE, "shim"), "-I", ref_src,
                  "-I", HERE, "-o", out, *srcs, *mine])
        built.append(out)
    return built


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-src", default=DEFAULT_REF_SRC)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    print(build_port(a.force))
    for p in build_ref(a.ref_src, a.force):
        print(p)


if __name__ == "__main__":
    sys.exit(main())
