"""The adler32 fused into the tensor-core epilogue (bf_form_beams_adler).

The checksum it returns must equal zlib's adler32 of the J it wrote, and the
reference's own checksums (arraysizes.cxx:54-57 and the seeded fixtures), for
both J layouts, host and device pointers, the chunked host-pointer pipeline
(several launches adding into one sum) and the dp4a fallback (separate pass).
"""
from __future__ import annotations

import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# partial last time tile (T % 64 != 0), ragged beams (B % 8 != 0), several
# beam passes, partial last K stage
SHAPES = [
    (64, 1, 64, 2, 8),
    (48, 2, 24, 2, 12),
    (80, 2, 72, 2, 40),
    (96, 2, 520, 2, 200),
    (256, 3, 512, 2, 128),
    (1024, 4, 512, 2, 64),
]


def _want(bflib, oracle, d, E, A, G, j_layout):
    od = oracle.Dims(d.ntimes, d.nfrequencies, d.ndishes, d.npolarizations, d.nbeams)
    J = oracle.form_beams(od, E, A, G)
    return oracle.J_to_J2(od, J) if j_layout == "j2" else J


@pytest.mark.parametrize("j_layout", ["linear", "j2"])
@pytest.mark.parametrize("shape", SHAPES)
def test_fused_adler_host_pointers(bflib, oracle, shape, j_layout):
    d = bflib.Dims(*shape)
    E, A, G = bflib.seeded_host_inputs(d, sum(shape))
    J = np.zeros(d.jsize, np.uint8)
    got = bflib.form_beams_adler(d, J, E, A, G, j_layout=j_layout)
    assert bflib.last_kernel() == "tensor"
    np.testing.assert_array_equal(J, _want(bflib, oracle, d, E, A, G, j_layout))
    assert got == zlib.adler32(J.tobytes())


@pytest.mark.parametrize("j_layout", ["linear", "j2"])
def test_fused_adler_device_pointers(bflib, cuda, oracle, j_layout):
    d = bflib.Dims(512, 3, 512, 2, 96)
    E, A, G = bflib.seeded_host_inputs(d, 21)
    Jd = cuda.full((d.jsize,), 0x5A, dtype=cuda.uint8, device="cuda")
    got = bflib.form_beams_adler(d, Jd, cuda.from_numpy(E).cuda(), cuda.from_numpy(A).cuda(),
                                 cuda.from_numpy(G).cuda(), j_layout=j_layout)
    J = Jd.cpu().numpy()
    np.testing.assert_array_equal(J, _want(bflib, oracle, d, E, A, G, j_layout))
    assert got == zlib.adler32(J.tobytes())


@pytest.mark.parametrize("j_layout", ["linear", "j2"])
def test_fused_adler_chunked_host_path(bflib, oracle, monkeypatch, j_layout):
    """Time chunks of 64 on three streams: every launch adds into the same sums
    with byte positions counted from the start of the whole J."""
    monkeypatch.setenv("BF_HOST_CHUNK_BYTES", str(64 * 4 * 512 * 2))
    d = bflib.Dims(1024, 4, 512, 2, 96)
    E, A, G = bflib.seeded_host_inputs(d, 22)
    J = np.zeros(d.jsize, np.uint8)
    got = bflib.form_beams_adler(d, J, E, A, G, j_layout=j_layout)
    np.testing.assert_array_equal(J, _want(bflib, oracle, d, E, A, G, j_layout))
    assert got == zlib.adler32(J.tobytes())


def test_fused_adler_simt_fallback(bflib, oracle):
    d = bflib.Dims(80, 2, 72, 2, 40)
    E, A, G = bflib.seeded_host_inputs(d, 23)
    bflib.set_kernel("simt")
    try:
        J = np.zeros(d.jsize, np.uint8)
        got = bflib.form_beams_adler(d, J, E, A, G)
        assert bflib.last_kernel() == "simt"
    finally:
        bflib.set_kernel("auto")
    np.testing.assert_array_equal(J, _want(bflib, oracle, d, E, A, G, "linear"))
    assert got == zlib.adler32(J.tobytes())


def test_fused_adler_reference_checksums(bflib, cuda, golden):
    """The reference's own checksums: its seeded outputs and the setup()
    pattern at t=32, f=32, b=128 (0xab69dfee, arraysizes.cxx:57) and at the
    production shape t=32768, f=16, b=96 (0x27303ea9, arraysizes.cxx:54)."""
    from oracle import oracle as O

    g, _ = golden
    for rec in g["seeded"]:
        d = bflib.Dims(rec["T"], rec["F"], rec["D"], rec["P"], rec["B"])
        E, A, G = bflib.seeded_host_inputs(d, rec["seed"])
        J = np.zeros(d.jsize, np.uint8)
        assert bflib.form_beams_adler(d, J, E, A, G) == rec["adler32"], rec
    for shape, want in (((32, 32, 512, 2, 128), 0xAB69DFEE), ((32768, 16, 512, 2, 96), 0x27303EA9)):
        d = bflib.Dims(*shape)
        E, A, G = O.setup_pattern(O.Dims(*shape))
        Jd = cuda.empty((d.jsize,), dtype=cuda.uint8, device="cuda")
        got = bflib.form_beams_adler(d, Jd, cuda.from_numpy(E).cuda(), cuda.from_numpy(A).cuda(),
                                     cuda.from_numpy(G).cuda())
        assert got == want, shape


def test_fused_adler_empty_problem(bflib):
    d = bflib.Dims(0, 1, 8, 2, 8)
    z = np.zeros(0, np.uint8)
    assert bflib.form_beams_adler(d, z, z, np.zeros(d.asize, np.uint8), np.zeros(d.gsize, np.float32)) == 1
