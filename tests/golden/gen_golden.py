"""Generate tests/golden/reference_vectors.json from the REFERENCE ITSELF.

Runs the reference's own sequential oracles -- cpuApsep (src/main.cu:102-113)
and cpuPSE (src/bench_spt_le.cu:24-35), compiled from the reference sources
by oracle/build_ref.py -- on the reference's own test inputs:

  * the structured small cases of src/main.cu:181-199 (inputs and outputs
    stored in full);
  * the random stress loops of src/main.cu:246-252 (std::mt19937 seeds
    42/43 with 500 trials of n <= 4096, seeds 100/101 with 200 trials of
    n <= 131072): per trial the length and the SHA-256 of the int32
    little-endian output;
  * the SPT "<" / "<=" distribution cases of src/bench_spt_le.cu:93-127 at
    the harness sizes 1000003, 513, 512, 511, 1 (and the full 2^25 for the
    cheap closed-form cases): SHA-256 of the output plus a few samples.

The inputs are regenerated from the same PRNG streams by oracle/ (no
reference needed at test time), so the fixtures pin the oracle restatement
and the CUDA engine to the reference's behaviour.

Usage: python tests/golden/gen_golden.py   (needs the reference tree)
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_vectors.json")


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<i4").tobytes()).hexdigest()


def main() -> int:
    if not oracle.ref_available():
        print("reference CPU oracle unavailable; cannot regenerate fixtures")
        return 1
    doc = {"generator": "tests/golden/gen_golden.py",
           "oracle": "reference cpuApsep (src/main.cu:102-113) and cpuPSE "
                     "(src/bench_spt_le.cu:24-35) compiled by oracle/build_ref.py",
           "hash": "sha256 of int32 little-endian output"}

    small = []
    for label, a in oracle.main_small_cases():
        small.append({"label": label, "input": a.tolist(),
                      "expected": oracle.ref_apse(a).tolist()})
    doc["main_small_cases"] = {"source": "src/main.cu:181-222", "cases": small}

    stress = []
    for seed, trials, max_n in ((42, 500, 4096), (43, 500, 4096),
                                (100, 200, 131072), (101, 200, 131072)):
        rows = []
        for a in oracle.main_stress_inputs(seed, trials, max_n):
            rows.append([int(a.shape[0]), sha(oracle.ref_apse(a))])
        stress.append({"seed": seed, "trials": trials, "max_n": max_n,
                       "trials_n_sha256": rows})
    doc["main_stress"] = {"source": "src/main.cu:145-175,246-252",
                          "value_mod": 1000000, "runs": stress}

    dist = []
    for name in oracle.SPT_LE_CASES:
        sizes = [1000003, 513, 512, 511, 1]
        if name in ("all-equal", "descending", "ascending", "dup2", "dup16"):
            sizes = [oracle.SPT_LE_FULL_N] + sizes
        full = oracle.gen_spt_le_case(name, max(sizes))
        for n in sizes:
            a = full[:n]
            for le in (False, True):
                r = oracle.ref_apse(a, le)
                idx = sorted({0, n // 3, n // 2, n - 1})
                dist.append({"case": name, "n": n, "le": le, "sha256": sha(r),
                             "samples": [[i, int(r[i])] for i in idx]})
    doc["spt_le_cases"] = {"source": "src/bench_spt_le.cu:93-127",
                           "full_n": oracle.SPT_LE_FULL_N, "entries": dist}

    with open(OUT, "w") as f:
        json.dump(doc, f, separators=(",", ":"))
        f.write("\n")
    print("wrote", OUT, os.path.getsize(OUT), "bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
