"""The C-ABI library on the CPU: it loads, exports every declared symbol, and
its host-only entry points behave; no compute call needs a GPU here."""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _header_symbols():
    text = open(os.path.join(ROOT, "include", "beamform.h")).read()
    return set(re.findall(r"^BF_API\s+[^(]*?\b(\w+)\s*\(", text, flags=re.M))


def test_header_and_package_agree(bflib):
    assert _header_symbols() == set(bflib.EXPORTED_SYMBOLS)


def test_library_exports_every_symbol(bflib):
    L = ctypes.CDLL(bflib.LIB_PATH)
    for name in _header_symbols():
        assert hasattr(L, name), name


def test_every_binding_declares_its_arguments(bflib):
    """Without argtypes ctypes passes Python ints as 32-bit C ints, which cuts
    64-bit addresses; every entry point the package binds declares them."""
    L = bflib.lib()
    for name in bflib.EXPORTED_SYMBOLS:
        assert getattr(L, name).argtypes is not None, name


def test_status_strings(bflib):
    L = bflib.lib()
    for code in range(0, 9):
        assert L.bf_status_string(code)
    assert L.bf_status_string(999) == b"unknown status"


def test_form_beams_before_set_dims(bflib):
    # A fresh process: form_beams() without bf_set_dims() reports NOT_CONFIGURED.
    import subprocess
    import sys

    code = (
        "import numpy as np, beamforming_gb300 as bf\n"
        "J=np.zeros(8,np.uint8); E=np.zeros(8,np.uint8); A=np.zeros(8,np.uint8); G=np.zeros(8,np.float32)\n"
        "L=bf.lib(); L.form_beams(J.ctypes.data,E.ctypes.data,A.ctypes.data,G.ctypes.data)\n"
        "print(L.bf_last_status())\n"
    )
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, check=True)
    assert r.stdout.strip() == str(bflib.ERR_NOT_CONFIGURED)


def test_invalid_arguments(bflib):
    L = bflib.lib()
    d = bflib.Dims(-1, 1, 1, 2, 1).c()
    assert L.bf_set_dims(ctypes.byref(d)) == bflib.ERR_INVALID_ARGUMENT
    assert L.bf_set_dims(None) == bflib.ERR_INVALID_ARGUMENT
    assert L.bf_set_kernel(7) == bflib.ERR_INVALID_ARGUMENT
    assert L.bf_set_kernel(4) == bflib.ERR_INVALID_ARGUMENT
    assert L.bf_set_kernel(3) == 0  # the 4-multiply SIMT form
    assert L.bf_set_kernel(0) == 0
    d = bflib.Dims(4, 1, 8, 2, 8).c()
    assert L.bf_form_beams_ex(ctypes.byref(d), None, None, None, None, 0, None) == bflib.ERR_INVALID_ARGUMENT
    J = np.zeros(64, np.uint8)
    assert L.bf_form_beams_ex(ctypes.byref(d), J.ctypes.data, J.ctypes.data, J.ctypes.data, J.ctypes.data, 5, None) == (
        bflib.ERR_INVALID_ARGUMENT
    )
    # empty problem: nothing to do, no device needed
    d0 = bflib.Dims(0, 1, 8, 2, 8).c()
    assert L.bf_form_beams_ex(ctypes.byref(d0), None, None, None, None, 0, None) == bflib.OK
    out = ctypes.c_uint32()
    assert L.bf_adler32_device(None, 0, ctypes.byref(out), None) == bflib.OK and out.value == 1
    # the checksummed call wants somewhere to put the checksum; an empty problem's is 1
    assert L.bf_form_beams_adler(ctypes.byref(d0), None, None, None, None, 0, 0, 0, None, None) == (
        bflib.ERR_INVALID_ARGUMENT)
    assert L.bf_form_beams_adler(ctypes.byref(d0), None, None, None, None, 0, 0, 0, ctypes.byref(out), None) == bflib.OK
    assert out.value == 1
    # layouts are checked before any device work
    dl = bflib.Dims(16, 1, 128, 2, 8).c()
    assert L.bf_form_beams_layout(ctypes.byref(dl), J.ctypes.data, J.ctypes.data, J.ctypes.data, J.ctypes.data, 2, 0,
                                  0, None) == bflib.ERR_INVALID_ARGUMENT
    assert L.bf_form_beams_layout(ctypes.byref(dl), J.ctypes.data, J.ctypes.data, J.ctypes.data, J.ctypes.data, 1, 0,
                                  0, None) == bflib.ERR_UNSUPPORTED  # A2 needs 256 or 512 dishes
    # server entry points check their handles before touching a device
    h = ctypes.c_void_p()
    assert L.bf_server_create(ctypes.byref(h), None, None) == bflib.ERR_INVALID_ARGUMENT
    t = ctypes.c_int64()
    assert L.bf_server_submit(None, 0, 1, 16, None, 0, None, 0, ctypes.byref(t)) == bflib.ERR_INVALID_ARGUMENT
    assert L.bf_server_wait(None, 0, None) == bflib.ERR_INVALID_ARGUMENT
    assert L.bf_server_drain(None) == bflib.ERR_INVALID_ARGUMENT
    assert L.bf_server_destroy(None) == bflib.OK
    wall = ctypes.c_double()
    assert L.bf_server_replay(None, 0, None, None, None, 0, None, 0, None, 0, None, 0, None, None, None,
                              ctypes.byref(wall), None) == bflib.ERR_INVALID_ARGUMENT


@pytest.mark.parametrize("n", [0, 1, 7, 5551, 5552, 5553, 3 * 5552 + 11, (1 << 20) + 7])
def test_host_adler32_matches_zlib(bflib, n):
    """bf_adler32_host (no device) equals zlib's adler32 across the 5552-byte
    reduction blocks, on all-0xFF bytes (the largest sums) and random bytes."""
    import zlib

    rng = np.random.default_rng(n)
    for data in (np.full(n, 255, np.uint8), rng.integers(0, 256, n, dtype=np.uint8)):
        assert bflib.adler32_host(data) == zlib.adler32(data.tobytes())


def test_python_argument_checks(bflib):
    d = bflib.Dims(4, 1, 8, 2, 8)
    with pytest.raises(ValueError):
        bflib.form_beams_ex(d, np.zeros(3, np.uint8), np.zeros(d.esize, np.uint8), np.zeros(d.asize, np.uint8),
                            np.zeros(d.gsize, np.float32))
    with pytest.raises(ValueError):
        bflib.form_beams(np.zeros(d.jsize, np.int8), np.zeros(d.esize, np.uint8), np.zeros(d.asize, np.uint8),
                         np.zeros(d.gsize, np.float32))


def test_host_generator_matches_oracle(bflib, oracle):
    for n, seed, sid in [(1, 0, 0), (13, 1, 1), (4096, 2, 0), (100003, 3, 1)]:
        x = np.empty(n, np.uint8)
        bflib.fill_random_host(x, seed, sid)
        np.testing.assert_array_equal(x, oracle.fill_random(n, seed, sid))


@pytest.mark.parametrize("shape", [(2048, 16, 512, 2, 96), (7, 3, 5, 2, 3), (1, 84, 512, 2, 96), (1, 16, 1024, 2, 512)])
def test_host_gains_match_oracle(bflib, oracle, shape):
    np.testing.assert_array_equal(bflib.gains(bflib.Dims(*shape)), oracle.gains(oracle.Dims(*shape)))


def test_no_device_reported(bflib):
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    d = bflib.Dims(16, 1, 8, 2, 8)
    E, A, G = bflib.seeded_host_inputs(d, 1)
    J = np.zeros(d.jsize, np.uint8)
    with pytest.raises(bflib.BeamformError) as ei:
        bflib.form_beams_ex(d, J, E, A, G)
    assert ei.value.status == bflib.ERR_NO_DEVICE


def test_every_entry_point_checks_its_arguments_before_the_device(bflib):
    """Null handles and pointers, and impossible sizes, are refused by every
    entry point without a device; empty work succeeds."""
    L = bflib.lib()
    E = bflib.ERR_INVALID_ARGUMENT
    h = ctypes.c_void_p()
    d = bflib.Dims(4, 1, 8, 2, 8).c()
    d0 = bflib.Dims(0, 1, 8, 2, 8).c()
    assert L.bf_weights_create(None, 1, 8, 8, None, None, 0, None) == E
    assert L.bf_weights_create(ctypes.byref(h), 0, 8, 8, None, None, 0, None) == E
    assert L.bf_weights_update(None, None, None, 0, None) == E
    assert L.bf_weights_destroy(None) == bflib.OK
    assert L.bf_form_beams_resident(None, 0, None, None, 16, None) == E
    assert L.bf_form_beams_noalloc(None, None, None, None, None, None) == E
    assert L.bf_form_beams_noalloc(ctypes.byref(d), None, None, None, None, None) == E
    assert L.bf_form_beams_noalloc(ctypes.byref(d0), None, None, None, None, None) == bflib.OK
    assert L.bf_batch_create(None, None, 0, None) == E
    assert L.bf_batch_run(None, None) == E
    assert L.bf_batch_info(None, None, None, None, None, None) == E
    assert L.bf_batch_shape(None, None, None, None, None, None, None, None) == E
    assert L.bf_batch_destroy(None) == bflib.OK
    assert L.bf_server_update_weights(None, None, None, 0) == E
    assert L.bf_server_stats_get(None, None) == E
    assert L.bf_fill_random_host(None, 4, 1, 0) == E
    assert L.bf_fill_random_host(None, 0, 1, 0) == bflib.OK
    assert L.bf_fill_random_device(None, 4, 1, 0, None) == E
    assert L.bf_gains_host(None, None) == E
    out = (ctypes.c_int * 12)()
    assert L.bf_plan_rings(0, 8, 0, 0, out) == E
    assert L.bf_plan_rings(512, 8, 0, 0, None) == E
    assert L.bf_plan_rings(512, 96, 0, 0, out) == bflib.OK
    assert L.bf_dp4a_peak(None, None) == E
    assert L.bf_tensor_peak(None, None) == E
