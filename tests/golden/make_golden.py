"""Generates the golden fixtures in this directory from the reference itself.

Run where the reference sources are present (after ``oracle/build_ref.sh``):

    python tests/golden/make_golden.py [group ...]

Groups: ``seeded``, ``full``, ``cases``, ``pattern`` (default: all).  Records of
the groups not named are kept from the existing golden.json.

For each shape it feeds seeded inputs (the workload generator: E stream 0,
A stream 1, G from setup()'s formula) to the reference's own form_beams
(cpu.cxx, compiled unmodified by oracle/build_ref.sh with that shape) and
records adler32(J); for small shapes it also stores J itself.  ``full`` does
the same for the full-size workloads (the t=32768 f=84 chunk and the wide
d=1024 b=512 array; adler32 only), ``cases`` for the named edge cases of
tests/golden/cases.py (huge gains, d=2048 extremes).  It also runs the stock
reference program (setup() pattern inputs) and records the checksum it
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
from tests.golden import cases as C  # noqa: E402

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
    (64, 2, 2048, 2, 96, 20),  # deepest dish count of the tensor-core path
]

# Full-size workloads, seeded: the single-GPU chunk (seed 1) and the wide
# array (seed 4).  adler32 only.
FULL = [
    (32768, 84, 512, 2, 96, 1),
    (16384, 16, 1024, 2, 512, 4),
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

GROUPS = ("seeded", "full", "cases", "pattern")


def shape_dir(T, F, D, P, B):
    return os.path.join(REF, f"{T}_{F}_{D}_{P}_{B}")


def run_ref(shape, E, A, G, tmp):
    """J from the reference's own form_beams (ref_io built for this shape)."""
    paths = [os.path.join(tmp, n) for n in ("E", "A", "G", "J")]
    E.tofile(paths[0])
    A.tofile(paths[1])
    G.astype(np.float32).tofile(paths[2])
    r = subprocess.run([os.path.join(shape_dir(*shape), "ref_io"), *paths], check=True, capture_output=True, text=True)
    J = np.fromfile(paths[3], dtype=np.uint8)
    for p in paths:
        os.remove(p)
    return J, float(r.stdout.strip() or 0.0)


def seeded_records(table, arrays, tmp, keep_arrays=True):
    recs = []
    for T, F, D, P, B, seed in table:
        dims = O.Dims(T, F, D, P, B)
        E, A, G = O.seeded_inputs(dims, seed)
        J, secs = run_ref((T, F, D, P, B), E, A, G, tmp)
        key = f"J_{T}_{F}_{D}_{P}_{B}_s{seed}"
        rec = {"T": T, "F": F, "D": D, "P": P, "B": B, "seed": seed, "adler32": O.adler32(J)}
        if keep_arrays and J.size <= 65536:
            arrays[key] = J
            rec["array"] = key
        recs.append(rec)
        print(key, hex(rec["adler32"]), f"{secs:.2f} s", flush=True)
    return recs


def case_records(arrays, tmp):
    recs = []
    for name in C.case_names():
        shape, E, A, G = C.make_case(name)
        J, _ = run_ref(shape, E, A, G, tmp)
        key = f"J_case_{name}"
        arrays[key] = J
        T, F, D, P, B = shape
        recs.append({"name": name, "T": T, "F": F, "D": D, "P": P, "B": B, "adler32": O.adler32(J), "array": key})
        print(key, hex(recs[-1]["adler32"]), flush=True)
    return recs


def pattern_records():
    recs = []
    for T, F, D, P, B in PATTERN:
        r = subprocess.run([os.path.join(shape_dir(T, F, D, P, B), "cpu")], capture_output=True, text=True)
        m = re.search(r"Checksum: 0x([0-9a-f]{8})", r.stdout)
        rec = {"T": T, "F": F, "D": D, "P": P, "B": B, "adler32": int(m.group(1), 16), "stock_exit": r.returncode}
        recs.append(rec)
        print("pattern", T, F, D, P, B, hex(rec["adler32"]), r.returncode, flush=True)
    return recs


def main(argv):
    groups = argv or list(GROUPS)
    for g in groups:
        if g not in GROUPS:
            raise SystemExit(f"unknown group {g!r}; groups: {', '.join(GROUPS)}")
    path = os.path.join(HERE, "golden.json")
    npz = os.path.join(HERE, "golden_J.npz")
    out = {"generator": "tests/golden/make_golden.py"}
    arrays = {}
    if os.path.exists(path):
        with open(path) as fp:
            out.update(json.load(fp))
        arrays.update(dict(np.load(npz)))
    for g in groups:  # drop the stored arrays of the groups being regenerated
        for rec in out.get(g, []):
            arrays.pop(rec.get("array", ""), None)
    with tempfile.TemporaryDirectory() as tmp:
        if "seeded" in groups:
            out["seeded"] = seeded_records(SEEDED, arrays, tmp)
        if "full" in groups:
            out["full"] = seeded_records(FULL, arrays, tmp, keep_arrays=False)
        if "cases" in groups:
            out["cases"] = case_records(arrays, tmp)
    if "pattern" in groups:
        out["pattern"] = pattern_records()
    out = {k: out[k] for k in ("generator", "seeded", "full", "cases", "pattern") if k in out}
    with open(path, "w") as fp:
        json.dump(out, fp, indent=1)
    np.savez_compressed(npz, **arrays)


if __name__ == "__main__":
    main(sys.argv[1:])
