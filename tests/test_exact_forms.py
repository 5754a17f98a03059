"""The arithmetic of the exact dp4a kernel's Gauss form, checked exhaustively
on the CPU against the oracle's decoding:

* the Gauss identity (k1 - k2 = Ar Er - Ai Ei, k1 + k3 = Ar Ei + Ai Er, with
  k1 = Ar (Er + Ei), k2 = (Ar + Ai) Ei, k3 = (Ai - Ar) Er) for every pair of
  stored bytes, and every factor in int8 range (what dp4a multiplies);
* the byte-lane decode of four stored bytes at once (each lane computes a
  difference with a bias of 128 so that no lane borrows from the next),
  restated here as 32-bit integer arithmetic, for every byte value in every
  lane.
"""
from __future__ import annotations

import numpy as np


def _lanes_sub(v, s):
    return (((v | 0x80808080) - s) & 0xFFFFFFFF) ^ 0x80808080


def _planes(w):
    hi, lo = (w >> 4) & 0x0F0F0F0F, w & 0x0F0F0F0F
    return (_lanes_sub(hi, 0x08080808), _lanes_sub(lo, 0x08080808), _lanes_sub(hi + lo, 0x10101010),
            _lanes_sub(lo, hi))


def _lane(w, i):
    b = (w >> (8 * i)) & 0xFF
    return b - 256 if b >= 128 else b


def test_gauss_identity_over_all_byte_pairs(oracle):
    parts = np.array([oracle.decode(b) for b in range(256)], dtype=np.int64)  # (re, im) of each stored byte
    ar, ai = parts[:, 0][:, None], parts[:, 1][:, None]  # A byte (rows)
    er, ei = parts[:, 0][None, :], parts[:, 1][None, :]  # E byte (columns)
    for f in (ar, ai, er, ei, er + ei, ar + ai, ai - ar):
        assert f.min() >= -128 and f.max() <= 127
    k1, k2, k3 = ar * (er + ei), (ar + ai) * ei, (ai - ar) * er
    assert np.array_equal(k1 - k2, ar * er - ai * ei)  # cpu.cxx:33
    assert np.array_equal(k1 + k3, ar * ei + ai * er)  # cpu.cxx:34
    assert max(abs(k).max() for k in (k1, k2, k3)) <= 128  # int32 sums exact for D < 2^24


def test_byte_lane_decode_matches_the_oracle(oracle):
    dec = [oracle.decode(b) for b in range(256)]
    rng = np.random.default_rng(5)
    for lane in range(4):
        for b in range(256):
            fill = [int(x) for x in rng.integers(0, 256, 4)]
            fill[lane] = b
            w = sum(x << (8 * i) for i, x in enumerate(fill))
            re, im, sm, df = _planes(w)
            for i in range(4):
                r, m = dec[fill[i]]
                assert (_lane(re, i), _lane(im, i), _lane(sm, i), _lane(df, i)) == (r, m, r + m, m - r)


def test_polarization_split_selectors():
    """__byte_perm(w0, w1, 0x6420 / 0x7531) on the bytes [d p0, d p1, d+1 p0,
    d+1 p1] [d+2 p0, ...] gives the four dishes of one polarization."""
    def perm(x, y, sel):
        b = [(x >> (8 * i)) & 255 for i in range(4)] + [(y >> (8 * i)) & 255 for i in range(4)]
        return sum(b[(sel >> (4 * i)) & 7] << (8 * i) for i in range(4))

    w0, w1 = 0x11100100, 0x31302120  # byte = 16 * dish + polarization
    assert perm(w0, w1, 0x6420) == 0x30201000
    assert perm(w0, w1, 0x7531) == 0x31211101
