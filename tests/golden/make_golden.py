"""Generate golden vectors from the reference's own code (run in a tree where
the reference sources are present).

The reference's standalone headers src/math/AliasTable.h and
src/math/SobolMatrices256x32.h are compiled into oracle/_ref/libzglref.so
(oracle/build_oracle.py).  This script records:

* alias tables that AliasTable::build<int32_t> produces for seeded pdf vectors
  (the light-selection table of Scene.cpp:243), and
* the SHA-256 of the 256x32 Sobol generator matrices plus their first and last
  columns of a few dimensions,

into tests/golden/reference_tables.json, so that tests on machines without the
reference tree still pin the product's tables to the reference's outputs.
"""
from __future__ import annotations

import hashlib
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

OUT = Path(__file__).resolve().parent / "reference_tables.json"


def pdf_cases():
    rng = np.random.default_rng(2024)
    cases = {
        "uniform4": np.ones(4, np.float32),
        "one_heavy": np.array([100.0, 1.0, 1.0, 1.0, 1.0], np.float32),
        "with_zero": np.array([0.0, 2.0, 0.0, 5.0, 1.0, 0.0], np.float32),
        "single": np.array([3.0], np.float32),
        "random64": rng.random(64).astype(np.float32),
        "lognormal257": rng.lognormal(0.0, 2.0, 257).astype(np.float32),
        "areas_cornell": np.array([0.299 * 7.5 + 0.587 * 7.5 + 0.114 * 7.5] * 2, np.float32),
    }
    return cases


def main() -> int:
    ref = oracle.ref_lib()
    if ref is None:
        print("reference tree not present; nothing generated")
        return 1
    out = {"alias": {}, "sobol": {}}
    for name, pdf in pdf_cases().items():
        n = pdf.size
        alias = np.zeros(n, np.int32)
        prob = np.zeros(n, np.float32)
        ref.ref_alias_build(pdf.ctypes.data, n, alias.ctypes.data, prob.ctypes.data)
        out["alias"][name] = {"pdf": pdf.view(np.uint32).tolist(), "alias": alias.tolist(),
                              "prob_bits": prob.view(np.uint32).tolist()}
    mats = np.zeros(256 * 32, np.uint32)
    ref.ref_sobol_matrices(mats.ctypes.data, mats.size)
    out["sobol"] = {"sha256": hashlib.sha256(mats.tobytes()).hexdigest(),
                    "dims": {str(d): mats[d * 32:(d + 1) * 32].tolist() for d in (0, 1, 2, 7, 100, 255)}}
    OUT.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {OUT}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
