"""The oracle pinned against the reference: golden checksums, encoding
asserts, adler32, and byte-for-byte fixtures made by the reference itself."""
from __future__ import annotations

import zlib

import numpy as np
import pytest


# icomplex4.hxx:63-74 -- the reference's static_asserts on the encoding
@pytest.mark.parametrize(
    "re,im,data",
    [(1, 2, 0x9A), (-1, 2, 0x7A), (1, -2, 0x96), (-1, -2, 0x76)],
)
def test_ucomplex4_static_asserts(oracle, re, im, data):
    assert oracle.encode(re, im) == data
    assert oracle.decode(data) == (re, im)


def test_ucomplex4_roundtrip_all_bytes(oracle):
    for byte in range(256):
        re, im = oracle.decode(byte)
        assert -8 <= re <= 7 and -8 <= im <= 7
        assert oracle.encode(re, im) == byte
        # offset-binary storage: high nibble = re + 8, low nibble = im + 8
        assert byte >> 4 == re + 8 and byte & 15 == im + 8


@pytest.mark.parametrize("n", [0, 1, 7, 100, 5552, 5553, 65536, 1 << 20])
def test_adler32_matches_zlib(oracle, n):
    data = np.random.default_rng(n).integers(0, 256, n, dtype=np.uint8)
    assert oracle.adler32(data) == zlib.adler32(data.tobytes())


def test_adler32_all_ff(oracle):
    data = np.full(1 << 16, 0xFF, dtype=np.uint8)
    assert oracle.adler32(data) == zlib.adler32(data.tobytes())


def test_seeded_generator_uniform_nibbles(oracle):
    x = oracle.fill_random(1 << 20, 3, 0)
    hi, lo = np.bincount(x >> 4, minlength=16), np.bincount(x & 15, minlength=16)
    expect = (1 << 20) / 16
    assert np.all(np.abs(hi - expect) < 0.02 * expect)
    assert np.all(np.abs(lo - expect) < 0.02 * expect)
    assert not np.array_equal(oracle.fill_random(4096, 3, 0), oracle.fill_random(4096, 3, 1))
    # prefix-stable: the first n bytes do not depend on the total length
    assert np.array_equal(oracle.fill_random(1001, 9, 0)[:999], oracle.fill_random(999, 9, 0))


def _pattern_cases(golden):
    g, _ = golden
    return g["pattern"]


# Reference checksums arraysizes.cxx:54-57 (the first four) plus the stock
# program's printed checksums for the other shapes.
PATTERN_REF = {
    (32768, 16, 512, 2, 96): 0x27303EA9,
    (32768, 32, 512, 2, 128): 0x4DE6498F,
    (32768, 32, 512, 2, 96): 0xC4FB6A4C,
    (32, 32, 512, 2, 128): 0xAB69DFEE,
}


@pytest.mark.parametrize(
    "shape",
    [
        (32, 32, 512, 2, 128),
        (2048, 16, 512, 2, 96),
        (8, 32, 512, 2, 128),
        (1, 32, 512, 2, 128),
        (32768, 16, 512, 2, 96),
        (32768, 32, 512, 2, 96),
        (32768, 32, 512, 2, 128),
    ],
)
def test_pattern_goldens(oracle, golden, shape):
    """setup() pattern inputs (arraysizes.cxx:8-52) give the reference's checksums."""
    g, _ = golden
    rec = next(r for r in g["pattern"] if (r["T"], r["F"], r["D"], r["P"], r["B"]) == shape)
    if shape in PATTERN_REF:
        assert rec["adler32"] == PATTERN_REF[shape]
    dims = oracle.Dims(*shape)
    E, A, G = oracle.setup_pattern(dims)
    J = oracle.form_beams(dims, E, A, G)
    assert oracle.adler32(J) == rec["adler32"]


def test_seeded_fixtures(oracle, golden):
    """Seeded inputs: the oracle reproduces the reference's own output bytes."""
    g, arrays = golden
    for rec in g["seeded"]:
        dims = oracle.Dims(rec["T"], rec["F"], rec["D"], rec["P"], rec["B"])
        E, A, G = oracle.seeded_inputs(dims, rec["seed"])
        J = oracle.form_beams(dims, E, A, G)
        assert oracle.adler32(J) == rec["adler32"], rec
        if "array" in rec:
            np.testing.assert_array_equal(J, arrays[rec["array"]])


def test_full_size_fixtures(oracle, golden):
    """The full single-GPU chunk (t=32768 f=84 d=512 b=96, seed 1) and the
    wide array (t=16384 f=16 d=1024 b=512, seed 4): the oracle's adler32 over
    all of J equals the one the reference's own cpu.cxx gave."""
    g, _ = golden
    for rec in g["full"]:
        dims = oracle.Dims(rec["T"], rec["F"], rec["D"], rec["P"], rec["B"])
        E, A, G = oracle.seeded_inputs(dims, rec["seed"])
        J = oracle.form_beams(dims, E, A, G)
        assert oracle.adler32(J) == rec["adler32"], rec
        del E, J


def test_case_fixtures(oracle, golden):
    """Edge cases (huge and non-finite gains; d=2048 extremes): the oracle
    gives the reference's own bytes."""
    from tests.golden import cases as C

    g, arrays = golden
    assert sorted(r["name"] for r in g["cases"]) == sorted(C.case_names())
    for rec in g["cases"]:
        shape, E, A, G = C.make_case(rec["name"])
        J = oracle.form_beams(oracle.Dims(*shape), E, A, G)
        np.testing.assert_array_equal(J, arrays[rec["array"]], err_msg=rec["name"])


def _narrow_model(g, raw):
    """int(lrint(g * raw)) clamped to [-7, 7] as the reference's x86-64 build does it."""
    with np.errstate(invalid="ignore", over="ignore"):
        x = np.float32(g) * np.float32(raw)
    if not np.isfinite(x) or abs(float(x)) >= 2.0**63:
        return 0
    v = int(np.rint(np.float64(x)))  # a float32 this large is an integer; half-even below
    v = (v + 2**31) % 2**32 - 2**31
    return max(-7, min(7, v))


def test_requant_narrowing(oracle):
    """cpu.cxx:38 narrows lrint's long to int before the clamp: products from
    2^31 up keep their low 32 bits, and NaN / inf / >= 2^63 give 0."""
    dims = oracle.Dims(16, 1, 64, 2, 16)
    E, A, _ = oracle.seeded_inputs(dims, 8)
    G = np.array([2.0**26, -2.0**26, 3.0e7, -5.5e8, 2.0**40 + 2.0**20, 1.0e18, 6.0e18, 1.0e19,
                  np.inf, -np.inf, np.nan, 2.0**31, 0.75, -1.0e-3, 2.0**-140, 1.0e30], np.float32)
    J = oracle.form_beams(dims, E, A, G)
    wrapped = 0
    for b in range(dims.nbeams):
        for p in range(2):
            for t in range(dims.ntimes):
                re, im = oracle.raw_sum(dims, E, A, b, 0, p, t)
                want = oracle.encode(_narrow_model(G[b], re), _narrow_model(G[b], im))
                assert J[(b * 2 + p) * dims.ntimes + t] == want, (b, p, t, G[b], re, im)
                with np.errstate(invalid="ignore", over="ignore"):
                    x = float(np.float32(G[b]) * np.float32(re))
                wrapped += 2.0**31 <= abs(x) < 2.0**63 and _narrow_model(G[b], re) != int(np.sign(x)) * 7
    assert wrapped > 0  # the narrowing changed some results


def test_raw_sum_matches_requant(oracle):
    dims = oracle.Dims(16, 2, 40, 2, 8)
    E, A, G = oracle.seeded_inputs(dims, 4)
    J = oracle.form_beams(dims, E, A, G)
    for b, f, p, t in [(0, 0, 0, 0), (7, 1, 1, 15), (3, 1, 0, 9)]:
        re, im = oracle.raw_sum(dims, E, A, b, f, p, t)
        g = np.float32(G[f * dims.nbeams + b])
        jre = int(np.clip(np.rint(g * np.float32(re)), -7, 7))
        jim = int(np.clip(np.rint(g * np.float32(im)), -7, 7))
        assert J[((b * dims.nfrequencies + f) * dims.npolarizations + p) * dims.ntimes + t] == oracle.encode(jre, jim)


def test_J_to_J2_layout(oracle):
    dims = oracle.Dims(5, 2, 8, 2, 3)
    J = np.arange(dims.jsize, dtype=np.uint8)
    J2 = oracle.J_to_J2(dims, J)
    T, F, P, B = 5, 2, 2, 3
    for b in range(B):
        for f in range(F):
            for p in range(P):
                for t in range(T):
                    assert J2[((b * F + f) * T + t) * P + p] == J[((b * F + f) * P + p) * T + t]


@pytest.mark.parametrize("D", [256, 512])
def test_A_to_A2_layout(oracle, D):
    """Every (f, b, c, d) lands in the nibble A2linear(f, b, c, d') names, d'
    the dish order of cuda4.cu:1468-1494 (arraysizes.hxx:125)."""
    F, B = 2, 3
    rng = np.random.default_rng(5)
    A = rng.integers(0, 256, F * B * D, dtype=np.uint8)
    dims = oracle.Dims(16, F, D, 2, B)
    A2 = oracle.A_to_A2(dims, A)

    def signed4(x):
        return x - 16 if x >= 8 else x

    perm = set()
    for f in range(F):
        for b in range(B):
            for d in range(D):
                dp = (d & 0x100) | ((d & 63) << 2) | ((d >> 6) & 3)
                perm.add(dp)
                a = int(A[(f * B + b) * D + d]) ^ 0x88
                for c, want in ((0, signed4(a >> 4)), (1, signed4(a & 15))):
                    i = dp + D * (c + 2 * (b + B * f))
                    byte = int(A2[i // 2]) ^ 0x88
                    got = signed4(byte >> 4) if i % 2 else signed4(byte & 15)
                    assert got == want
    assert perm == set(range(D))  # a permutation of the dishes


def test_reference_gpu_kernel_covers_only_its_launch():
    """The reference GPU kernel's launch (4 x 8 x 12 threads per frequency,
    cuda.cu:290-296) covers nbeams only when nbeams / 8 is a multiple of 12;
    the loader refuses every other shape whether or not a cubin exists."""
    from oracle import ref_gpu

    for shape in [(2048, 16, 512, 2, 128), (2048, 16, 512, 2, 64), (2048, 16, 512, 2, 100), (2048, 16, 500, 2, 96),
                  (2044, 16, 512, 2, 96), (2048, 16, 512, 1, 96)]:
        assert not ref_gpu.available(*shape), shape
