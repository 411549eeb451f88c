"""Generate tests/golden/*.json from the reference's own golden files.

The reference ships two golden population files (PETSc binary, 128x128 D2Q9,
2 components, natural order):
  tests/bubble_2D/reference_solution/fi001.dat       (SRT, isotropy 4)
  tests/bubble_2D_hots/reference_solution/fi001.dat  (MRT, isotropy 10)
For each, this script records the SHA-256 of the big-endian float64 payload,
per-(direction, component) sums and 4096 values at seeded positions, so tests
can check bit-exactness without the 2.3 MB files.  Run it where the
reference tree is available:  python tests/golden/make_golden.py
"""
import hashlib
import json
import os

import numpy as np

REF = os.environ.get("TAXILA_REFERENCE", "/root/reference")  # the reference checkout
HERE = os.path.dirname(os.path.abspath(__file__))
CASES = {
    "bubble_2D": "tests/bubble_2D/reference_solution/fi001.dat",
    "bubble_2D_hots": "tests/bubble_2D_hots/reference_solution/fi001.dat",
}


def digest(values):
    """SHA-256 of float64 values serialised big-endian, as PETSc writes them."""
    return hashlib.sha256(np.asarray(values, dtype=">f8").tobytes()).hexdigest()


def main():
    for name, rel in CASES.items():
        raw = open(os.path.join(REF, rel), "rb").read()
        head = np.frombuffer(raw[:8], dtype=">i4")
        vals = np.frombuffer(raw[8:], dtype=">f8").astype(np.float64)
        assert head[0] == 1211214 and head[1] == vals.size
        rng = np.random.default_rng(20240607)
        idx = np.sort(rng.choice(vals.size, 4096, replace=False))
        rec = {
            "source": "reference " + rel,
            "n": int(vals.size),
            "sha256_be": digest(vals),
            "sums_per_dof": vals.reshape(-1, 18).sum(axis=0).tolist(),
            "sample_index": idx.tolist(),
            "sample_value": vals[idx].tolist(),
        }
        with open(os.path.join(HERE, name + "_fi001.json"), "w") as f:
            json.dump(rec, f)
        print(name, rec["sha256_be"])


if __name__ == "__main__":
    main()
