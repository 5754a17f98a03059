"""The host-pointer pipeline with J in pinned host memory: a drain kernel
behind each time chunk writes the chunk's row segments straight into the
caller's J (no copy at the end).  The bytes must equal the oracle's for both
J layouts, a partial last chunk, both kernels and the checksummed call."""
from __future__ import annotations

import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pinned(cuda, n):
    return cuda.empty(n, dtype=cuda.uint8, pin_memory=True).numpy()


def _oracle_J(oracle, d, E, A, G, j_layout):
    od = oracle.Dims(d.ntimes, d.nfrequencies, d.ndishes, d.npolarizations, d.nbeams)
    J = oracle.form_beams(od, E, A, G)
    return oracle.J_to_J2(od, J) if j_layout == "j2" else J


@pytest.mark.parametrize("kernel", ["tensor", "simt"])
@pytest.mark.parametrize("T", [1024, 1040])
@pytest.mark.parametrize("j_layout", ["linear", "j2"])
def test_pinned_J_drained_per_chunk(bflib, cuda, oracle, monkeypatch, j_layout, T, kernel):
    # 256 times per chunk: T = 1040 ends with a chunk of 16 times
    monkeypatch.setenv("BF_HOST_CHUNK_BYTES", str(256 * 4 * 512 * 2))
    d = bflib.Dims(T, 4, 512, 2, 96)
    E, A, G = bflib.seeded_host_inputs(d, T + (1 if j_layout == "j2" else 0))
    J = _pinned(cuda, d.jsize)
    J[:] = 0x5A
    bflib.set_kernel(kernel)
    try:
        bflib.form_beams_layout(d, J, E, A, G, j_layout=j_layout)
        assert bflib.last_kernel() == kernel
    finally:
        bflib.set_kernel("auto")
    np.testing.assert_array_equal(J, _oracle_J(oracle, d, E, A, G, j_layout))


def test_pinned_J_with_checksum(bflib, cuda, oracle, monkeypatch):
    monkeypatch.setenv("BF_HOST_CHUNK_BYTES", str(256 * 4 * 512 * 2))
    d = bflib.Dims(1024, 4, 512, 2, 96)
    E, A, G = bflib.seeded_host_inputs(d, 31)
    J = _pinned(cuda, d.jsize)
    got = bflib.form_beams_adler(d, J, E, A, G)
    np.testing.assert_array_equal(J, _oracle_J(oracle, d, E, A, G, "linear"))
    assert got == zlib.adler32(J.tobytes())


def test_pinned_and_pageable_J_agree(bflib, cuda):
    """The drained path and the copy-at-the-end path give the same bytes on
    the same inputs (pageable J takes the latter)."""
    d = bflib.Dims(2048, 16, 512, 2, 96)
    E, A, G = bflib.seeded_host_inputs(d, 0)
    Jp = _pinned(cuda, d.jsize)
    Jh = np.zeros(d.jsize, np.uint8)
    bflib.form_beams_ex(d, Jp, E, A, G)
    bflib.form_beams_ex(d, Jh, E, A, G)
    np.testing.assert_array_equal(Jp, Jh)


def test_pinned_J_with_unaligned_rows_falls_back(bflib, cuda, oracle, monkeypatch):
    """Rows of T = 200 bytes are not a multiple of 16: the drain cannot write
    them with 16-byte stores, so J is copied out once at the end (the dp4a
    kernel takes this T)."""
    monkeypatch.setenv("BF_HOST_CHUNK_BYTES", str(64 * 2 * 64 * 2))
    d = bflib.Dims(200, 2, 64, 2, 24)
    E, A, G = bflib.seeded_host_inputs(d, 41)
    J = _pinned(cuda, d.jsize)
    J[:] = 0x5A
    bflib.form_beams_ex(d, J, E, A, G)
    np.testing.assert_array_equal(J, _oracle_J(oracle, d, E, A, G, "linear"))


@pytest.mark.parametrize("kernel", ["tensor", "simt"])
@pytest.mark.parametrize("T", [1024, 1040])
@pytest.mark.parametrize("j_layout", ["linear", "j2"])
def test_pageable_J_pipelined(bflib, cuda, oracle, monkeypatch, j_layout, T, kernel):
    """J in pageable memory (the drop-in case: the reference's main passes
    std::vector storage) through the chunked host pipeline: J leaves in one
    copy after the last chunk; the bytes equal the oracle's, twice in a row,
    including a 16-time last chunk."""
    monkeypatch.setenv("BF_HOST_CHUNK_BYTES", str(256 * 4 * 512 * 2))
    d = bflib.Dims(T, 4, 512, 2, 96)
    E, A, G = bflib.seeded_host_inputs(d, T + 7 + (1 if j_layout == "j2" else 0))
    expect = _oracle_J(oracle, d, E, A, G, j_layout)
    bflib.set_kernel(kernel)
    try:
        for _ in range(2):
            J = np.full(d.jsize, 0x5A, np.uint8)  # pageable
            bflib.form_beams_layout(d, J, E, A, G, j_layout=j_layout)
            assert bflib.last_kernel() == kernel
            np.testing.assert_array_equal(J, expect)
    finally:
        bflib.set_kernel("auto")


def test_pageable_J_with_checksum(bflib, cuda, oracle, monkeypatch):
    monkeypatch.setenv("BF_HOST_CHUNK_BYTES", str(256 * 4 * 512 * 2))
    d = bflib.Dims(1024, 4, 512, 2, 96)
    E, A, G = bflib.seeded_host_inputs(d, 41)
    J = np.zeros(d.jsize, np.uint8)
    got = bflib.form_beams_adler(d, J, E, A, G)
    expect = _oracle_J(oracle, d, E, A, G, "linear")
    np.testing.assert_array_equal(J, expect)
    assert got == zlib.adler32(expect.tobytes())
