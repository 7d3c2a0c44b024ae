"""The POY-side stub file shown in INTEGRATION.md compiles against POY's own
headers (seq.h, cm.h) and include/poyalgn.h, with the caml header shim used
by the oracle build. Skipped where the POY sources are absent."""
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from build_oracle import DEFAULT_REF_SRC  # noqa: E402


@pytest.mark.skipif(not os.path.isfile(os.path.join(DEFAULT_REF_SRC, "seq.h")),
                    reason="POY sources absent")
def test_integration_stubs_compile(tmp_path):
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```c\n(.*?)```", text, re.S)
    assert blocks
    src = tmp_path / "stubs.c"
    src.write_text(blocks[0])
    subprocess.run(["gcc", "-fsyntax-only", "-std=gnu11", "-fgnu89-inline", "-Werror",
                    "-Wimplicit-function-declaration",
                    "-I", os.path.join(ROOT, "oracle", "shim"), "-I", DEFAULT_REF_SRC,
                    "-I", os.path.join(ROOT, "include"), str(src)], check=True)
