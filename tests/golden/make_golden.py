"""Generates the golden fixtures in this directory from the reference itself.

Run where the reference sources are present (after ``oracle/build_ref.sh``):

    python tests/golden/make_golden.py

For each shape it feeds seeded inputs (the workload generator: E stream 0,
A stream 1, G from setup()'s formula) to the reference's own form_beams
(cpu.cxx, compiled unmodified by oracle/build_ref.sh with that shape) and
records adler32(J); for small shapes it also stores J itself.  It also runs the
stock reference program (setup() pattern inputs) and records the checksum it
prints.  The tests compare the oracle and the CUDA path against these files;
nothing at test time runs the reference.
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")

# (T, F, D, P, B, seed); J is stored in full when it is at most 64 KiB.
SEEDED = [
    (64, 2, 64, 2, 8, 11),
    (40, 3, 32, 2, 16, 12),
    (33, 2, 48, 2, 24, 13),
    (8, 1, 32, 2, 8, 14),
    (1, 1, 1, 2, 1, 15),
    (7, 3, 5, 2, 3, 16),
    (16, 2, 32, 1, 8, 17),
    (256, 1, 512, 2, 128, 18),
    (128, 2, 1024, 2, 512, 19),
    (2048, 16, 512, 2, 96, 0),  # plain-beamform workload, seed 0
]

# Stock programs (setup() pattern); the first four carry the reference's own
# checksums (arraysizes.cxx:54-57).
PATTERN = [
    (32768, 16, 512, 2, 96),
    (32768, 32, 512, 2, 96),
    (32768, 32, 512, 2, 128),
    (32, 32, 512, 2, 128),
    (2048, 16, 512, 2, 96),
    (8, 32, 512, 2, 128),
    (1, 32, 512, 2, 128),
]


def shape_dir(T, F, D, P, B):
    return os.path.join(REF, f"{T}_{F}_{D}_{P}_{B}")


def main():
    out = {"generator": "tests/golden/make_golden.py", "seeded": [], "pattern": []}
    arrays = {}
    with tempfile.TemporaryDirectory() as tmp:
        for T, F, D, P, B, seed in SEEDED:
            dims = O.Dims(T, F, D, P, B)
            E, A, G = O.seeded_inputs(dims, seed)
            paths = [os.path.join(tmp, n) for n in ("E", "A", "G", "J")]
            E.tofile(paths[0])
            A.tofile(paths[1])
            G.tofile(paths[2])
            subprocess.run([os.path.join(shape_dir(T, F, D, P, B), "ref_io"), *paths], check=True, capture_output=True)
            J = np.fromfile(paths[3], dtype=np.uint8)
            key = f"J_{T}_{F}_{D}_{P}_{B}_s{seed}"
            rec = {"T": T, "F": F, "D": D, "P": P, "B": B, "seed": seed, "adler32": O.adler32(J)}
            if J.size <= 65536:
                arrays[key] = J
                rec["array"] = key
            out["seeded"].append(rec)
            print(key, hex(rec["adler32"]))
    for T, F, D, P, B in PATTERN:
        r = subprocess.run([os.path.join(shape_dir(T, F, D, P, B), "cpu")], capture_output=True, text=True)
        m = re.search(r"Checksum: 0x([0-9a-f]{8})", r.stdout)
        rec = {"T": T, "F": F, "D": D, "P": P, "B": B, "adler32": int(m.group(1), 16), "stock_exit": r.returncode}
        out["pattern"].append(rec)
        print("pattern", T, F, D, P, B, hex(rec["adler32"]), r.returncode)
    with open(os.path.join(HERE, "golden.json"), "w") as fp:
        json.dump(out, fp, indent=1)
    np.savez_compressed(os.path.join(HERE, "golden_J.npz"), **arrays)


if __name__ == "__main__":
    main()
