"""Named input cases for the golden fixtures (test infrastructure).

Each case is a shape plus a deterministic construction of E, A and G.  The
fixture generator (make_golden.py) feeds them to the reference's own
form_beams (cpu.cxx, compiled unmodified) and stores its output; the tests
rebuild the same inputs from this module and compare the CUDA path with the
stored bytes.  The cases cover the edges of the accepted domain:

* ``big_gain``: gains whose products with the raw sums reach 2^31 and beyond.
  cpu.cxx:38 narrows lrint's 64-bit result to int before it clamps, so such a
  product keeps only its low 32 bits; NaN, infinite and |G*raw| >= 2^63
  products give 0 (the x86-64 lrint result LONG_MIN narrowed).
* ``extreme_d2048_*``: the deepest dish count the tensor-core path takes
  (2048) with inputs that drive |raw J| and the weight row sums to their
  largest values (a row sum of -2^15 for all_min).
"""
from __future__ import annotations

import os
import sys

import numpy as np

_ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
if _ROOT not in sys.path:
    sys.path.insert(0, _ROOT)

from oracle import oracle as O  # noqa: E402

BIG_GAIN_SHAPE = (256, 1, 512, 2, 128)
D2048_SHAPE = (64, 2, 2048, 2, 96)
EXTREME_KINDS = ("all_min", "all_max", "min_max", "alternating")


def big_gains(n: int) -> np.ndarray:
    """n gains (n >= 16): magnitudes 2^-12 .. 2^70 with non-round mantissas,
    both signs, plus zero, +-inf, NaN, the largest float and a subnormal."""
    g = np.empty(n, np.float32)
    special = [0.0, np.inf, -np.inf, np.nan, np.finfo(np.float32).max, -np.finfo(np.float32).max, 1e-42, 2.0**31]
    g[: len(special)] = np.array(special, np.float32)
    rng = np.random.default_rng(2031)
    m = n - len(special)
    expo = np.linspace(-12, 70, m)
    mant = rng.uniform(1.0, 2.0, m)
    sign = np.where(np.arange(m) % 2 == 0, 1.0, -1.0)
    g[len(special):] = (sign * mant * np.exp2(expo)).astype(np.float32)
    return g


def extreme_EA(dims: O.Dims, kind: str) -> tuple[np.ndarray, np.ndarray]:
    E = np.empty(dims.esize, np.uint8)
    A = np.empty(dims.asize, np.uint8)
    if kind == "all_min":  # every nibble -8: weight row sums reach -16 D = -2^15 at D = 2048
        E[:] = 0x00
        A[:] = 0x00
    elif kind == "all_max":  # every nibble +7
        E[:] = 0xFF
        A[:] = 0xFF
    elif kind == "min_max":  # E all -8, A re -8 im +7
        E[:] = 0x00
        A[:] = 0x0F
    elif kind == "alternating":
        E[0::2], E[1::2] = 0x0F, 0xF0
        A[0::3], A[1::3], A[2::3] = 0x00, 0xFF, 0x0F
    else:
        raise ValueError(kind)
    return E, A


def extreme_gains(dims: O.Dims) -> np.ndarray:
    """Gains that spread the largest |raw| = 2 * 64 * D over the clamp range,
    both signs, with zero and exact-half ties."""
    rng = np.random.default_rng(dims.ndishes)
    base = np.float32(7.5 / (2 * 64 * dims.ndishes))
    G = (rng.uniform(-2, 2, dims.gsize).astype(np.float32) * base).astype(np.float32)
    G[0], G[1], G[2] = 0.0, np.float32(0.5 / 128), np.float32(-1.5 / 256)
    return G


def case_names() -> list[str]:
    return ["big_gain"] + [f"extreme_d2048_{k}" for k in EXTREME_KINDS]


def make_case(name: str) -> tuple[tuple[int, int, int, int, int], np.ndarray, np.ndarray, np.ndarray]:
    """(shape, E, A, G) of a named case."""
    if name == "big_gain":
        dims = O.Dims(*BIG_GAIN_SHAPE)
        E, A, _ = O.seeded_inputs(dims, 23)
        return BIG_GAIN_SHAPE, E, A, big_gains(dims.gsize)
    if name.startswith("extreme_d2048_"):
        dims = O.Dims(*D2048_SHAPE)
        E, A = extreme_EA(dims, name[len("extreme_d2048_"):])
        return D2048_SHAPE, E, A, extreme_gains(dims)
    raise ValueError(name)
