"""Generate the golden vectors in tests/golden/ from the reference's own Mugs
oracle (gpu/Mugs.cc, built unmodified into oracle/_ref by oracle/Makefile
with the single-process MPI stand-in).

    python tests/golden/make_golden.py

Each case stores the shape, the initial state (reference formula
gpu/main.cc:18, or integer seed), compute flag, shares, and the resulting
field (padded DArray layout, all ranks) plus its SHA-256.  The reference has
no periodic mode, so every case is non-periodic (MPI_PROC_NULL outside the
rank grid).  Needs the reference sources; the fixtures then pin the oracle
everywhere else.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

CASES = [
    # name, (lx,ly,lz,mx,my,mz,n), init, seed, compute, shares
    ("c1_ref", (1, 1, 1, 4, 4, 4, 5), "ref", 0, True, 5),
    ("c1_int", (1, 1, 1, 4, 4, 4, 5), "int", 1, True, 5),
    ("c1_ref_nocompute", (1, 1, 1, 4, 4, 4, 5), "ref", 0, False, 3),
    ("ranks_2x2x1_int", (2, 2, 1, 2, 3, 2, 4), "int", 7, True, 3),
    ("ranks_2x2x1_ref", (2, 2, 1, 2, 3, 2, 4), "ref", 0, True, 3),
    ("ranks_3x1x2_int_nocompute", (3, 1, 2, 2, 1, 3, 6), "int", 11, False, 2),
    ("ranks_2x2x2_n2_int", (2, 2, 2, 1, 2, 1, 2), "int", 3, True, 4),
    ("single_n8_ref", (1, 1, 1, 3, 2, 2, 8), "ref", 0, True, 2),
]


def main() -> None:
    O.build()
    if not O.ref_available():
        sys.exit("the reference's Mugs (oracle/_ref) is not built: reference sources missing")
    index = []
    for name, shape, init, seed, compute, shares in CASES:
        s = O.Shape(*shape, periodic=False)
        u0 = O.init_ref(s) if init == "ref" else O.init_int(s, seed)
        out = O.ref_mugs_share(s, u0.copy(), compute, shares)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), out=out)
        index.append({"name": name, "shape": list(shape), "init": init, "seed": seed, "compute": compute,
                      "shares": shares, "sha256": hashlib.sha256(out.tobytes()).hexdigest()})
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump({"generator": "reference gpu/Mugs.cc via oracle/_ref", "cases": index}, fh, indent=1)
    print(f"wrote {len(index)} cases")


if __name__ == "__main__":
    main()
