"""Regenerate the generated fixtures in tests/golden/ (run from the repo root).

validate_points.npy   -- the 7,500 points of the reference's randomized validation test
                         (test/lbvh_test.cu:396-409), drawn with libstdc++'s mt19937 and
                         uniform_real_distribution<float> exactly as that test draws them.
validate_fixture.json -- the brute-force minimum-image neighbor counts for those points
                         (rcut 1, test/lbvh_test.cu:458-490), as a per-point checksum.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
import oracle as O  # noqa: E402


def main():
    L = np.array([20.0, 15.0, 25.0], np.float32)
    P = O.gen_validate_points(7500, L, 42)
    np.save(os.path.join(HERE, "validate_points.npy"), P)
    ref = O.brute_count(P, 1.0, P, L)
    fx = {
        "_about": "brute-force minimum-image counts (incl. self) for validate_points.npy, rcut 1",
        "pairs": int(ref.sum()),
        "max": int(ref.max()),
        "weighted_checksum": int((ref.astype(np.uint64) * np.arange(1, len(ref) + 1, dtype=np.uint64)).sum()),
    }
    with open(os.path.join(HERE, "validate_fixture.json"), "w") as f:
        json.dump(fx, f, indent=1)
    print(fx)


if __name__ == "__main__":
    main()
