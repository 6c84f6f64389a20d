"""The public headers as a C caller of the reference would use them: a C99
program (tests/c_abi/c_caller.c) including every header in
include/pyrsgm/ that declares C functions, compiled with gcc, linked
against libpyrsgm_gb300.so and run (it only makes calls that need no GPU)."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

from pyrsgm_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cuda_include() -> str | None:
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


def test_headers_compile_and_link_as_c(tmp_path):
    gcc, inc = shutil.which("gcc"), _cuda_include()
    if not gcc or not inc:
        pytest.skip("gcc or the CUDA headers not found")
    exe = str(tmp_path / "c_caller")
    lib_dir = os.path.dirname(_native.LIB_PATH)
    cmd = [gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-Wno-unused-parameter",
           os.path.join(ROOT, "tests", "c_abi", "c_caller.c"), "-o", exe,
           "-I" + os.path.join(ROOT, "include"), "-I" + inc,
           "-L" + lib_dir, "-lpyrsgm_gb300", "-Wl,-rpath," + lib_dir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, str(tmp_path / "x.pgm")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
