"""Parity of the CUDA path with the oracle and the reference's own outputs.

Every comparison is bit-exact (integer and byte work); all GPU calls go
through the C ABI of libbeamform.so.
"""
from __future__ import annotations

import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(torch, x):
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def run_gpu(bf, torch, dims, E, A, G, kernel="auto"):
    """One pass on device buffers through bf_form_beams_ex; returns J (host)."""
    bf.set_kernel(kernel)
    try:
        Jd = torch.full((dims.jsize,), 0x5A, dtype=torch.uint8, device="cuda")
        bf.form_beams_ex(dims, Jd, _dev(torch, E), _dev(torch, A), _dev(torch, G))
        bf.stream_status()
        return Jd.cpu().numpy()
    finally:
        bf.set_kernel("auto")


def oracle_dims(oracle, d):
    return oracle.Dims(d.ntimes, d.nfrequencies, d.ndishes, d.npolarizations, d.nbeams)


# Shapes the tensor-core kernel takes (P = 2, D % 8 == 0, T % 16 == 0), including
# ragged beams (B % 8 != 0), several beam passes (B > 128), a partial last K
# stage (D % 64 != 0) and a partial last time tile (T % 64 != 0).
TC_SHAPES = [
    (64, 1, 64, 2, 8),
    (16, 1, 8, 2, 8),
    (128, 2, 512, 2, 96),
    (256, 3, 512, 2, 128),
    (48, 2, 24, 2, 12),
    (80, 2, 72, 2, 40),
    (64, 1, 1024, 2, 512),
    (96, 2, 520, 2, 200),
    (336, 5, 512, 2, 16),
    (1024, 4, 512, 2, 64),
]


def _random_tc_shapes(n=40, seed=20261204):
    """Seeded shapes across every layout the tensor-core kernel picks: beam
    counts 1-300 (passes of 8-96 beams: two CTAs per SM, two unpack groups
    with the W forwarder, one group; ragged beams and several passes), dish
    counts 8-2048 (partial last K stage), 16-512 times (partial last time
    tile), 1-3 frequencies; sized so that the oracle finishes each in well
    under a second."""
    rng = np.random.default_rng(seed)
    shapes = []
    while len(shapes) < n:
        D = int(rng.integers(1, 257)) * 8
        B = int(rng.integers(1, 301))
        T = int(rng.integers(1, 33)) * 16
        F = int(rng.integers(1, 4))
        if T * F * 2 * B * D <= 4e7:
            shapes.append((T, F, D, 2, B))
    return shapes


@pytest.mark.parametrize("shape", _random_tc_shapes())
def test_random_shapes_tensor_vs_oracle(bflib, cuda, oracle, shape):
    d = bflib.Dims(*shape)
    E, A, G = bflib.seeded_host_inputs(d, sum(shape))
    J = run_gpu(bflib, cuda, d, E, A, G, "tensor")
    np.testing.assert_array_equal(J, oracle.form_beams(oracle_dims(oracle, d), E, A, G), err_msg=str(shape))


@pytest.mark.parametrize("shape", TC_SHAPES)
@pytest.mark.parametrize("kernel", ["tensor", "simt", "simt4"])
def test_seeded_shapes_match_oracle(bflib, cuda, oracle, shape, kernel):
    d = bflib.Dims(*shape)
    E, A, G = bflib.seeded_host_inputs(d, 100 + sum(shape))
    J = run_gpu(bflib, cuda, d, E, A, G, kernel)
    assert bflib.last_kernel() == kernel
    Jo = oracle.form_beams(oracle_dims(oracle, d), E, A, G)
    np.testing.assert_array_equal(J, Jo)


# Shapes only the SIMT kernel takes: odd times, odd dishes, one polarization.
SIMT_SHAPES = [(1, 1, 1, 2, 1), (7, 3, 5, 2, 3), (33, 2, 48, 2, 24), (16, 2, 32, 1, 8), (40, 3, 30, 2, 17)]


@pytest.mark.parametrize("shape", SIMT_SHAPES)
def test_odd_shapes_auto_dispatch(bflib, cuda, oracle, shape):
    d = bflib.Dims(*shape)
    E, A, G = bflib.seeded_host_inputs(d, 7)
    J = run_gpu(bflib, cuda, d, E, A, G, "auto")
    assert bflib.last_kernel() == "simt"
    want = oracle.form_beams(oracle_dims(oracle, d), E, A, G)
    np.testing.assert_array_equal(J, want)
    J4 = run_gpu(bflib, cuda, d, E, A, G, "simt4")  # the 4-multiply form
    assert bflib.last_kernel() == "simt4"
    np.testing.assert_array_equal(J4, want)


def test_tensor_kernel_refuses_odd_shape(bflib, cuda):
    d = bflib.Dims(7, 3, 5, 2, 3)
    E, A, G = bflib.seeded_host_inputs(d, 7)
    with pytest.raises(bflib.BeamformError) as ei:
        run_gpu(bflib, cuda, d, E, A, G, "tensor")
    assert ei.value.status == bflib.ERR_UNSUPPORTED


def test_reference_fixtures(bflib, cuda, golden):
    """The reference's own output bytes (compiled cpu.cxx on seeded inputs)."""
    g, arrays = golden
    for rec in g["seeded"]:
        d = bflib.Dims(rec["T"], rec["F"], rec["D"], rec["P"], rec["B"])
        E, A, G = bflib.seeded_host_inputs(d, rec["seed"])
        for kernel in ("auto", "simt"):
            J = run_gpu(bflib, cuda, d, E, A, G, kernel)
            assert zlib.adler32(J.tobytes()) == rec["adler32"], (rec, kernel)
            if "array" in rec:
                np.testing.assert_array_equal(J, arrays[rec["array"]])


def test_pattern_golden_small(bflib, cuda):
    """setup() pattern at t=32, f=32, d=512, b=128: checksum 0xab69dfee (arraysizes.cxx:57)."""
    from oracle import oracle as O

    d = bflib.Dims(32, 32, 512, 2, 128)
    E, A, G = O.setup_pattern(O.Dims(32, 32, 512, 2, 128))
    for kernel in ("tensor", "simt"):
        J = run_gpu(bflib, cuda, d, E, A, G, kernel)
        assert zlib.adler32(J.tobytes()) == 0xAB69DFEE, kernel


# setup() pattern shapes with the reference's checksums (arraysizes.cxx:54-57:
# 0x27303ea9, 0xc4fb6a4c, 0x4de6498f) and the ones its program printed here
PATTERN_SHAPES = [
    (32768, 16, 512, 2, 96),
    (32768, 32, 512, 2, 96),
    (32768, 32, 512, 2, 128),
    (2048, 16, 512, 2, 96),
    (8, 32, 512, 2, 128),
    (1, 32, 512, 2, 128),
]


@pytest.mark.parametrize("shape", PATTERN_SHAPES)
def test_pattern_goldens(bflib, cuda, golden, shape):
    """setup() pattern inputs give the reference's checksums (t = 8 and 1 run on
    the dp4a kernel, the others on the tensor cores; b = 128 in two passes)."""
    from oracle import oracle as O

    g, _ = golden
    rec = next(r for r in g["pattern"] if (r["T"], r["F"], r["D"], r["P"], r["B"]) == shape)
    d = bflib.Dims(*shape)
    E, A, G = O.setup_pattern(O.Dims(*shape))
    J = run_gpu(bflib, cuda, d, E, A, G)
    assert bflib.last_kernel() == ("tensor" if shape[0] % 16 == 0 else "simt")
    assert zlib.adler32(J.tobytes()) == rec["adler32"]


def test_plain_beamform_workload_drop_in(bflib, cuda, golden):
    """t=2048 f=16 d=512 b=96 seed 0 through the drop-in form_beams(J, E, A, G) on host arrays."""
    g, _ = golden
    rec = next(r for r in g["seeded"] if (r["T"], r["F"], r["D"], r["B"], r["seed"]) == (2048, 16, 512, 96, 0))
    d = bflib.Dims(2048, 16, 512, 2, 96)
    E, A, G = bflib.seeded_host_inputs(d, 0)
    J = np.zeros(d.jsize, np.uint8)
    bflib.set_dims(d)
    bflib.form_beams(J, E, A, G)
    assert bflib.last_kernel() == "tensor"
    assert zlib.adler32(J.tobytes()) == rec["adler32"]
    # host-pointer explicit call gives the same bytes
    J2 = np.zeros_like(J)
    bflib.form_beams_ex(d, J2, E, A, G)
    np.testing.assert_array_equal(J, J2)


@pytest.mark.parametrize("shape", [(1000, 3, 512, 2, 96), (400, 5, 30, 2, 17), (1024, 2, 64, 2, 8)])
def test_host_pointer_pipeline(bflib, cuda, oracle, shape, monkeypatch):
    """Host-pointer calls pipelined over time chunks on several streams (small
    chunks forced here; a ragged last chunk; tensor and SIMT shapes); the bytes
    equal the oracle's."""
    monkeypatch.setenv("BF_HOST_CHUNK_BYTES", str(64 * 1024))
    d = bflib.Dims(*shape)
    E, A, G = bflib.seeded_host_inputs(d, 31)
    J = np.full(d.jsize, 0x5A, np.uint8)
    bflib.form_beams_ex(d, J, E, A, G)
    np.testing.assert_array_equal(J, oracle.form_beams(oracle_dims(oracle, d), E, A, G))


def _extreme_inputs(d, kind):
    E = np.empty(d.esize, np.uint8)
    A = np.empty(d.asize, np.uint8)
    if kind == "all_min":  # every nibble -8
        E[:] = 0x00
        A[:] = 0x00
    elif kind == "all_max":  # every nibble +7
        E[:] = 0xFF
        A[:] = 0xFF
    elif kind == "min_max":
        E[:] = 0x00
        A[:] = 0x0F  # re -8, im +7
    elif kind == "alternating":
        E[0::2], E[1::2] = 0x0F, 0xF0
        A[0::3], A[1::3], A[2::3] = 0x00, 0xFF, 0x0F
    elif kind == "zero":
        E[:] = 0x88
        A[:] = 0x88
    return E, A


@pytest.mark.parametrize("kind", ["all_min", "all_max", "min_max", "alternating", "zero"])
@pytest.mark.parametrize("D", [512, 1024, 2048])
def test_adversarial_extremes(bflib, cuda, oracle, kind, D):
    """Largest |raw J| (|sum| up to 2 * 64 * D) and every G sign: exactness of the tensor path."""
    d = bflib.Dims(128, 2, D, 2, 64)
    E, A = _extreme_inputs(d, kind)
    rng = np.random.default_rng(D)
    # gains spanning the clamp range, both signs, exact-half ties, zero
    base = np.float32(7.5 / (2 * 64 * D))
    G = (rng.uniform(-2, 2, d.gsize).astype(np.float32) * base).astype(np.float32)
    G[0], G[1], G[2] = 0.0, np.float32(0.5 / 128), np.float32(-1.5 / 256)
    for kernel in ("tensor", "simt", "simt4"):
        J = run_gpu(bflib, cuda, d, E, A, G, kernel)
        np.testing.assert_array_equal(J, oracle.form_beams(oracle_dims(oracle, d), E, A, G), err_msg=kernel)


def test_half_way_rounding(bflib, cuda, oracle):
    """G * raw landing exactly on .5 rounds half to even (lrint, cpu.cxx:38)."""
    d = bflib.Dims(64, 1, 64, 2, 16)
    E, A, G = bflib.seeded_host_inputs(d, 3)
    G[:] = np.float32(0.5) ** np.arange(1, 17, dtype=np.float32)
    for kernel in ("tensor", "simt", "simt4"):
        J = run_gpu(bflib, cuda, d, E, A, G, kernel)
        np.testing.assert_array_equal(J, oracle.form_beams(oracle_dims(oracle, d), E, A, G), err_msg=kernel)


@pytest.mark.parametrize("scale", [1e-4, 0.3, 7.0, 1e4])
def test_gain_ranges(bflib, cuda, oracle, scale):
    """Gains from tiny to huge, both signs: covers the packed 16-bit clamp
    (small |G| * |raw|) and the single-precision clamp (large) of the epilogue."""
    d = bflib.Dims(192, 3, 512, 2, 40)
    E, A, _ = bflib.seeded_host_inputs(d, 21)
    rng = np.random.default_rng(int(scale * 10) + 1)
    G = (rng.uniform(-1, 1, d.gsize) * scale).astype(np.float32)
    G[::7] = np.float32(0.0)
    for kernel in ("tensor", "simt", "simt4"):
        J = run_gpu(bflib, cuda, d, E, A, G, kernel)
        np.testing.assert_array_equal(J, oracle.form_beams(oracle_dims(oracle, d), E, A, G), err_msg=kernel)


def test_impulse(bflib, cuda, oracle):
    """cuda4.cu:1325-1412 impulse construction with a fixed seed: one nonzero
    A, E and G; J = G*A*E at one (b,f,p,t) and zero elsewhere."""
    rng = np.random.default_rng(42)
    d = bflib.Dims(256, 4, 512, 2, 96)
    for _ in range(4):
        b, f, t, p, dish = (int(rng.integers(0, n)) for n in (d.nbeams, d.nfrequencies, d.ntimes, 2, d.ndishes))
        while True:
            a = complex(int(rng.integers(-2, 3)), int(rng.integers(-2, 3)))
            e = complex(int(rng.integers(-2, 3)), int(rng.integers(-2, 3)))
            gv = int(rng.integers(-2, 3))
            j = gv * a * e
            if max(abs((a * e).real), abs((a * e).imag), abs(j.real), abs(j.imag)) <= 7:
                break
        E = np.full(d.esize, 0x88, np.uint8)
        A = np.full(d.asize, 0x88, np.uint8)
        G = np.zeros(d.gsize, np.float32)
        E[((t * d.nfrequencies + f) * d.ndishes + dish) * 2 + p] = oracle.encode(int(e.real), int(e.imag))
        A[(f * d.nbeams + b) * d.ndishes + dish] = oracle.encode(int(a.real), int(a.imag))
        G[f * d.nbeams + b] = gv
        expect = np.full(d.jsize, 0x88, np.uint8)
        expect[((b * d.nfrequencies + f) * 2 + p) * d.ntimes + t] = oracle.encode(int(j.real), int(j.imag))
        for kernel in ("tensor", "simt"):
            np.testing.assert_array_equal(run_gpu(bflib, cuda, d, E, A, G, kernel), expect, err_msg=kernel)


@pytest.mark.parametrize("n", [1, 100, 65535, 65536, 65537, 1 << 22, (1 << 22) + 12345])
def test_adler32_device(bflib, cuda, n):
    x = np.random.default_rng(n).integers(0, 256, n + 3, dtype=np.uint8)
    t = _dev(cuda, x)
    assert bflib.adler32_device(t[:n]) == zlib.adler32(x[:n].tobytes())
    # a start address that is not 16-byte aligned
    assert bflib.adler32_device(t[3:]) == zlib.adler32(x[3:].tobytes())


def test_device_generator_matches_host(bflib, cuda, oracle):
    for n, seed, sid in [(1, 0, 0), (13, 1, 1), (1 << 20, 2, 0), (100003, 3, 1)]:
        t = cuda.empty(n, dtype=cuda.uint8, device="cuda")
        bflib.fill_random_device(t, seed, sid)
        np.testing.assert_array_equal(t.cpu().numpy(), oracle.fill_random(n, seed, sid))


def test_resident_weights_and_refresh(bflib, cuda, oracle):
    """Device-resident weights; a refresh regenerates A from seed 4+k (the
    weight-refresh stream of the wide-array workload)."""
    F, B, D = 3, 96, 512
    for T in (256, 1024, 200):  # 200: not a multiple of 16 -> SIMT path with the resident weights
        d = bflib.Dims(T, F, D, 2, B)
        E = np.empty(d.esize, np.uint8)
        bflib.fill_random_host(E, 4, 0)
        G = bflib.gains(d)
        A0 = np.empty(d.asize, np.uint8)
        bflib.fill_random_host(A0, 4, 1)
        W = bflib.ResidentWeights(F, B, D, A0, G)
        Ed = _dev(cuda, E)
        for k in range(3):
            A = np.empty(d.asize, np.uint8)
            bflib.fill_random_host(A, 4 + k, 1)
            if k:
                W.update(_dev(cuda, A), _dev(cuda, G))
            Jd = cuda.empty(d.jsize, dtype=cuda.uint8, device="cuda")
            W.form_beams(Jd, Ed, T)
            bflib.stream_status()
            assert bflib.last_kernel() == ("tensor" if T % 16 == 0 else "simt")
            np.testing.assert_array_equal(Jd.cpu().numpy(), oracle.form_beams(oracle_dims(oracle, d), E, A, G))
        W.close()


def _full_record(golden, shape, seed):
    g, _ = golden
    return next(r for r in g["full"] if (r["T"], r["F"], r["D"], r["P"], r["B"], r["seed"]) == (*shape, seed))


def test_full_size_chunk_matches_reference(bflib, cuda, golden):
    """Full single-GPU chunk (t=32768 f=84 d=512 b=96, seed 1): the adler32 of
    all of J equals the reference cpu.cxx's on the same inputs, and the tensor
    and SIMT kernels agree on every byte."""
    shape = (32768, 84, 512, 2, 96)
    rec = _full_record(golden, shape, 1)
    d = bflib.Dims(*shape)
    E, A, G = bflib.seeded_host_inputs(d, 1)
    Ed, Ad, Gd = _dev(cuda, E), _dev(cuda, A), _dev(cuda, G)
    del E
    Jt = cuda.empty(d.jsize, dtype=cuda.uint8, device="cuda")
    Js = cuda.empty(d.jsize, dtype=cuda.uint8, device="cuda")
    bflib.set_kernel("tensor")
    bflib.form_beams_ex(d, Jt, Ed, Ad, Gd)
    bflib.set_kernel("simt")
    bflib.form_beams_ex(d, Js, Ed, Ad, Gd)
    bflib.set_kernel("auto")
    bflib.stream_status()
    assert bflib.adler32_device(Jt) == rec["adler32"]
    assert cuda.equal(Jt, Js)


@pytest.mark.parametrize("B", [16, 8, 12])
def test_narrowest_passes_large_chunk(bflib, cuda, B):
    """Passes of at most 16 beams run two CTAs per SM (t=32768 f=8 d=512, seed
    5: 4096 tiles, ~13 per CTA): the tensor and SIMT kernels agree on every
    byte, plain and through resident weights."""
    d = bflib.Dims(32768, 8, 512, 2, B)
    E, A, G = bflib.seeded_host_inputs(d, 5)
    Ed, Ad, Gd = _dev(cuda, E), _dev(cuda, A), _dev(cuda, G)
    Jt = cuda.full((d.jsize,), 0x5A, dtype=cuda.uint8, device="cuda")
    Js = cuda.full((d.jsize,), 0xA5, dtype=cuda.uint8, device="cuda")
    bflib.set_kernel("tensor")
    bflib.form_beams_ex(d, Jt, Ed, Ad, Gd)
    bflib.set_kernel("simt")
    bflib.form_beams_ex(d, Js, Ed, Ad, Gd)
    bflib.set_kernel("auto")
    bflib.stream_status()
    assert cuda.equal(Jt, Js)
    W = bflib.ResidentWeights(8, B, 512, Ad, Gd)
    try:
        Jr = cuda.full((d.jsize,), 0x33, dtype=cuda.uint8, device="cuda")
        W.form_beams(Jr, Ed, 32768)
        bflib.stream_status()
        assert cuda.equal(Jr, Js)
    finally:
        W.close()


def test_wide_array_matches_reference(bflib, cuda, golden):
    """Wide array (t=16384 f=16 d=1024 b=512, seed 4; six beam passes): adler32
    of all of J equals the reference cpu.cxx's, on both kernels."""
    shape = (16384, 16, 1024, 2, 512)
    rec = _full_record(golden, shape, 4)
    d = bflib.Dims(*shape)
    E, A, G = bflib.seeded_host_inputs(d, 4)
    Ed, Ad, Gd = _dev(cuda, E), _dev(cuda, A), _dev(cuda, G)
    Jd = cuda.empty(d.jsize, dtype=cuda.uint8, device="cuda")
    for kernel in ("tensor", "simt"):
        bflib.set_kernel(kernel)
        try:
            bflib.form_beams_ex(d, Jd, Ed, Ad, Gd)
            bflib.stream_status()
        finally:
            bflib.set_kernel("auto")
        assert bflib.adler32_device(Jd) == rec["adler32"], kernel


@pytest.mark.parametrize("name", ["big_gain", "extreme_d2048_all_min", "extreme_d2048_all_max",
                                  "extreme_d2048_min_max", "extreme_d2048_alternating"])
def test_edge_case_fixtures(bflib, cuda, golden, name):
    """The reference's own bytes at the edges of the domain: huge and
    non-finite gains (int narrowing of cpu.cxx:38 before the clamp) and the
    deepest dish count of the tensor-core path (d=2048) with extreme inputs
    (a weight row sum of -2^15, |raw| up to 2 * 64 * d)."""
    from tests.golden import cases as C

    g, arrays = golden
    rec = next(r for r in g["cases"] if r["name"] == name)
    shape, E, A, G = C.make_case(name)
    d = bflib.Dims(*shape)
    for kernel in ("tensor", "simt"):
        J = run_gpu(bflib, cuda, d, E, A, G, kernel)
        assert bflib.last_kernel() == kernel
        np.testing.assert_array_equal(J, arrays[rec["array"]], err_msg=kernel)


def test_wide_gains_resident_and_plain(bflib, cuda, oracle):
    """One frequency with huge gains beside ordinary ones: only that
    frequency takes the narrowing requantisation, in plain launches and with
    resident weights."""
    d = bflib.Dims(256, 3, 512, 2, 96)
    E, A, G = bflib.seeded_host_inputs(d, 44)
    G = G.copy()
    G[96:192] = np.float32(3.0e7) * np.linspace(-1, 1, 96, dtype=np.float32)  # frequency 1
    expect = oracle.form_beams(oracle_dims(oracle, d), E, A, G)
    np.testing.assert_array_equal(run_gpu(bflib, cuda, d, E, A, G, "tensor"), expect)
    W = bflib.ResidentWeights(3, 96, 512, A, G)
    try:
        Jd = cuda.empty(d.jsize, dtype=cuda.uint8, device="cuda")
        W.form_beams(Jd, _dev(cuda, E), 256)
        bflib.stream_status()
        np.testing.assert_array_equal(Jd.cpu().numpy(), expect)
    finally:
        W.close()


@pytest.mark.parametrize("B", [96, 32, 16])
def test_device_wait_timeout_reports_and_recovers(bflib, cuda, oracle, B):
    """A launch whose copies are never issued: its bounded waits expire, the
    call reports ERR_DEVICE_TIMEOUT, and the next launch is correct (b=96: one
    unpack group; b=32: two groups and the W forwarder; b=16: two CTAs per SM)."""
    d = bflib.Dims(128, 2, 512, 2, B)
    E, A, G = bflib.seeded_host_inputs(d, 9)
    bflib.set_test_stall(True)
    try:
        with pytest.raises(bflib.BeamformError) as ei:
            run_gpu(bflib, cuda, d, E, A, G, "tensor")
        assert ei.value.status == bflib.ERR_DEVICE_TIMEOUT
    finally:
        bflib.set_test_stall(False)
    J = run_gpu(bflib, cuda, d, E, A, G, "tensor")
    np.testing.assert_array_equal(J, oracle.form_beams(oracle_dims(oracle, d), E, A, G))


@pytest.mark.parametrize("shape", [(96, 2, 64, 2, 40), (64, 1, 128, 1, 33)])
def test_unaligned_operands_take_the_byte_path(bflib, cuda, oracle, shape):
    """E and A one byte off a 4-byte boundary (D % 4 == 0): the exact kernel
    decodes byte by byte instead of by words; auto dispatch goes there too."""
    d = bflib.Dims(*shape)
    E, A, G = bflib.seeded_host_inputs(d, 31)
    want = oracle.form_beams(oracle_dims(oracle, d), E, A, G)
    Eb = cuda.zeros(d.esize + 16, dtype=cuda.uint8, device="cuda")
    Ab = cuda.zeros(d.asize + 16, dtype=cuda.uint8, device="cuda")
    Ed, Ad = Eb[1:1 + d.esize], Ab[3:3 + d.asize]
    Ed.copy_(cuda.from_numpy(E))
    Ad.copy_(cuda.from_numpy(A))
    assert Ed.data_ptr() % 4 and Ad.data_ptr() % 4
    Gd = _dev(cuda, G)
    for kernel in ("simt", "simt4", "auto"):
        bflib.set_kernel(kernel)
        try:
            Jd = cuda.full((d.jsize,), 0x5A, dtype=cuda.uint8, device="cuda")
            bflib.form_beams_ex(d, Jd, Ed, Ad, Gd)
            bflib.stream_status()
        finally:
            bflib.set_kernel("auto")
        np.testing.assert_array_equal(Jd.cpu().numpy(), want, err_msg=kernel)
