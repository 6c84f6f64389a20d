"""Generate the golden fixtures that pin the CPU oracle: run every parity
case of tests/cases.py through the REFERENCE's own CUDA kernels (compiled
from its sources into oracle/_ref/*.fatbin, launched by
oracle/_build/libref_harness.so) on a GPU and store the outputs.

    python -m tests.golden.make_golden OUT.npz

Stored per case: disp16 (exact), conf (float32), a SHA-1 per row of disp32,
of the cost volume and of the aggregated volume (restricted to the columns
where the reference defines it), and the device adaptive-P2 table used.
pyrDown outputs on the reference test's pattern are stored whole.
"""
from __future__ import annotations

import hashlib
import sys

import numpy as np

from tests import _oracle, _runners, cases


def row_hashes(a: np.ndarray) -> np.ndarray:
    return np.array([np.frombuffer(hashlib.sha1(np.ascontiguousarray(r).tobytes()).digest(), np.uint8)
                     for r in a], dtype=np.uint8)


def main(path: str) -> None:
    import torch
    assert torch.cuda.is_available()
    _oracle.ref()
    out = {}
    for case in cases.SINGLE_SCALE + cases.LEVELS + cases.MATCHER:
        n = case["name"]
        r = _runners.run_ref(case)
        out[f"{n}/disp16"] = r["disp16"]
        out[f"{n}/conf"] = r["conf"]
        out[f"{n}/disp32_rows"] = row_hashes(r["disp32"])
        if "cost" in r:
            x0, x1 = r["acc_cols"]
            out[f"{n}/cost_rows"] = row_hashes(r["cost"])
            out[f"{n}/acc_rows"] = row_hashes(r["acc"][:, x0:x1])
        lut = _runners.device_lut(case)
        if lut is not None:
            out[f"{n}/p2lut"] = lut
        print(n, "valid px:", int((r["disp32"] > 0).sum()), flush=True)
    for w, h in cases.PYRDOWN:
        out[f"pyrdown_{w}x{h}"] = _runners.run_ref_pyrdown(cases.pyrdown_input(w, h))
    np.savez_compressed(path, **out)
    print("wrote", path)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "tests/golden/ref_golden.npz")
