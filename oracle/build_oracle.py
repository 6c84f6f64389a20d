"""Build recipe for the test oracles (test infrastructure only).

  oracle/_build/libsgm_oracle.so   CPU restatement (sgm_oracle.c), OpenMP
  oracle/_ref/sgm_kernels.fatbin   the reference's src/sgm_kernels.cu, unmodified,
  oracle/_ref/pyrdown.fatbin       and src/pyrdown.cu, compiled for sm_103a from
                                   the reference sources (only where the reference
                                   tree is present; the GPU machine uses these prebuilt
                                   device images)
  oracle/_build/libref_harness.so  ref_harness.cpp: loads the fatbins and replays
                                   the reference host launch schedule
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
# the reference source tree (only this build step reads it); PYRSGM_REFERENCE overrides
REFERENCE = os.environ.get("PYRSGM_REFERENCE", "/root/reference")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")

ORACLE_SO = os.path.join(BUILD, "libsgm_oracle.so")
HARNESS_SO = os.path.join(BUILD, "libref_harness.so")
SGM_FATBIN = os.path.join(REF_OUT, "sgm_kernels.fatbin")
PYR_FATBIN = os.path.join(REF_OUT, "pyrdown.fatbin")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: str, *deps: str) -> bool:
    return not os.path.exists(out) or os.path.getmtime(out) < max(os.path.getmtime(d) for d in deps)


def build_oracle() -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "sgm_oracle.c")
    hdr = os.path.join(HERE, "sgm_oracle.h")
    if _stale(ORACLE_SO, src, hdr):
        base = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", src, "-o", ORACLE_SO, "-lm"]
        try:
            _run(base[:1] + ["-fopenmp"] + base[1:])
        except RuntimeError:
            _run(base)  # no OpenMP runtime: single-threaded oracle
    return ORACLE_SO


def build_ref_fatbins() -> bool:
    """Compile the reference kernels (only where the reference tree exists)."""
    src_sgm = os.path.join(REFERENCE, "src", "sgm_kernels.cu")
    src_pyr = os.path.join(REFERENCE, "src", "pyrdown.cu")
    if not (os.path.exists(src_sgm) and os.path.exists(src_pyr)):
        return os.path.exists(SGM_FATBIN) and os.path.exists(PYR_FATBIN)
    os.makedirs(REF_OUT, exist_ok=True)
    nvcc = shutil.which("nvcc") or os.path.join(CUDA, "bin", "nvcc")
    inc = "-I" + os.path.join(REFERENCE, "include")
    for src, out in ((src_sgm, SGM_FATBIN), (src_pyr, PYR_FATBIN)):
        if _stale(out, src):
            _run([nvcc, "-fatbin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo",
                  inc, "-o", out, src])
    return True


def build_harness() -> str:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "ref_harness.cpp")
    if _stale(HARNESS_SO, src):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", src, "-o", HARNESS_SO,
              "-I" + os.path.join(CUDA, "include"), "-L" + os.path.join(CUDA, "lib64"), "-lcudart"])
    return HARNESS_SO


def build_all() -> dict:
    out = {"oracle": build_oracle(), "harness": build_harness(), "ref_fatbins": build_ref_fatbins()}
    return out


if __name__ == "__main__":
    print(build_all())
    sys.exit(0)
