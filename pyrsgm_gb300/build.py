"""Build the native library libpyrsgm_gb300.so in-tree (sm_103a only).

Each CUDA translation unit is compiled to an object under
pyrsgm_gb300/_build/ in parallel, then linked into
pyrsgm_gb300/libpyrsgm_gb300.so.  Objects are reused when newer than their
source and every header under csrc/ and include/.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libpyrsgm_gb300.so")
# the checked build (range checks in the kernels, a synchronous check after
# every launch): separate objects and library, loaded with PYRSGM_GB300_CHECKED=1
BUILD_CHECKED = os.path.join(PKG, "_build_checked")
LIB_CHECKED = os.path.join(PKG, "libpyrsgm_gb300_checked.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _headers() -> list[str]:
    out = []
    for d in (CSRC, os.path.join(ROOT, "include", "pyrsgm")):
        for f in os.listdir(d):
            if f.endswith((".h", ".cuh")):
                out.append(os.path.join(d, f))
    return out


def _sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _flags(checked: bool = False) -> list[str]:
    return ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O2,-Wall,-Wextra,-Wno-unused-parameter",
                   "-I" + CSRC, "-I" + os.path.join(ROOT, "include")] + (["-DPYRSGM_CHECKED=1"] if checked else [])


def _compile(src: str, hdr_mtime: float, verbose: bool, checked: bool = False) -> str:
    obj = os.path.join(BUILD_CHECKED if checked else BUILD, os.path.basename(src)[:-3] + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), hdr_mtime):
        return obj
    cmd = [nvcc(), "-c", src, "-o", obj] + _flags(checked)
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout.strip() or r.stderr.strip()):
        print(r.stdout + r.stderr, flush=True)
    return obj


def build(verbose: bool = False, jobs: int | None = None, checked: bool = False) -> str:
    """The library (and the CLI); checked=True builds the checked library instead."""
    out = LIB_CHECKED if checked else LIB
    os.makedirs(BUILD_CHECKED if checked else BUILD, exist_ok=True)
    hdr_mtime = max(os.path.getmtime(h) for h in _headers())
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdr_mtime, verbose, checked), srcs))
    if not (os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(o) for o in objs)):
        tmp = out + ".tmp"
        cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, out)
    if not checked:
        build_cli(hdr_mtime)
    return out


CLI_SRC = os.path.join(PKG, "cli", "stereo_pair.cpp")
CLI = os.path.join(PKG, "pyrsgm_stereo_pair")


def build_cli(hdr_mtime: float) -> str:
    """The headless stereo CLI, linked against the library (rpath to it)."""
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(os.path.getmtime(CLI_SRC), os.path.getmtime(LIB),
                                                             hdr_mtime):
        return CLI
    cmd = [nvcc(), "-O2", "-std=c++17", "-x", "cu", CLI_SRC, "-o", CLI + ".tmp", "-I" + os.path.join(ROOT, "include"),
           "-L" + PKG, "-lpyrsgm_gb300", "-Xlinker", "-rpath=" + PKG] + ARCH
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(CLI + ".tmp", CLI)
    return CLI


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, checked="--checked" in sys.argv))
