"""bf_form_beams_noalloc: the entry point for callers that cannot allocate
device memory (a real-time pipeline that sizes its device memory once at
start-up, or a framework that owns the memory pool).  It keeps its scratch in a
fixed 4 MiB device array, so it must give the same bytes as the regular
bf_form_beams_ex on every call, even though each call reuses the array the
previous call left behind.

This file sorts last so that a run stopping at the first failure has already
run every other test; it also passes alone in a fresh process.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call_noalloc(bf, torch, dims, J, E, A, G):
    d = dims.c()
    stream = torch.cuda.current_stream().cuda_stream
    return bf.lib().bf_form_beams_noalloc(
        ctypes.byref(d), J.data_ptr(), E.data_ptr(), A.data_ptr(), G.data_ptr(), stream
    )


def _inputs(bf, torch, dims, seed):
    E = torch.empty(dims.esize, dtype=torch.uint8, device="cuda")
    A = torch.empty(dims.asize, dtype=torch.uint8, device="cuda")
    bf.fill_random_device(E, seed, 0)
    bf.fill_random_device(A, seed, 1)
    G = torch.from_numpy(bf.gains(dims)).cuda()
    return E, A, G


def test_noalloc_matches_regular_entry_point_twice(bflib, cuda):
    bf, torch = bflib, cuda
    dims = bf.Dims(2048, 16, 512, 2, 96)  # plain-beamform workload: operand 3 MiB, fits the 4 MiB array
    cases = [_inputs(bf, torch, dims, seed) for seed in (0, 5)]
    outs = [torch.full((dims.jsize,), 0x5A, dtype=torch.uint8, device="cuda") for _ in cases]
    torch.cuda.synchronize()

    # two calls in a row, different inputs; the second must not see the first's scratch
    for (E, A, G), J in zip(cases, outs):
        assert _call_noalloc(bf, torch, dims, J, E, A, G) == bf.OK

    # a third call measured: it allocates nothing on the device
    free_before = torch.cuda.mem_get_info()[0]
    assert _call_noalloc(bf, torch, dims, outs[1], *cases[1]) == bf.OK
    assert torch.cuda.mem_get_info()[0] == free_before

    # the regular entry point on the same inputs gives the same bytes (exact)
    bf.set_kernel("tensor")
    try:
        for (E, A, G), J in zip(cases, outs):
            ref = torch.empty_like(J)
            bf.form_beams_ex(dims, ref, E, A, G)
            bf.stream_status()
            assert torch.equal(J, ref)
            assert bf.adler32_device(J) == bf.adler32_device(ref)
    finally:
        bf.set_kernel("auto")
    assert not torch.equal(outs[0], outs[1])


def test_noalloc_rejects_what_does_not_fit(bflib, cuda):
    bf, torch = bflib, cuda
    big = bf.Dims(64, 84, 512, 2, 96)  # 16.5 MB operand > 4 MiB
    E = torch.zeros(big.esize, dtype=torch.uint8, device="cuda")
    A = torch.zeros(big.asize, dtype=torch.uint8, device="cuda")
    G = torch.zeros(big.gsize, dtype=torch.float32, device="cuda")
    J = torch.zeros(big.jsize, dtype=torch.uint8, device="cuda")
    assert _call_noalloc(bf, torch, big, J, E, A, G) == bf.ERR_TOO_LARGE
    odd = bf.Dims(7, 1, 5, 2, 3)  # not a tensor-core shape
    assert _call_noalloc(bf, torch, odd, J, E, A, G) == bf.ERR_UNSUPPORTED
    assert not torch.any(J)
