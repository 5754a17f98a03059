"""The wide-array shape (d=1024, b=512: six beam passes of 88 beams over a
2048-byte K) against the oracle, and weight refresh inside the served loop:
chunks submitted between refreshes use the weights current at submission,
with no drain, every chunk exact."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

B, D = 512, 1024


def _weights(bflib, F, seed):
    d = bflib.Dims(16, F, D, 2, B)
    A = np.empty(d.asize, np.uint8)
    bflib.fill_random_host(A, seed, 1)
    return A, bflib.gains(d)


@pytest.mark.parametrize("kernel", ["tensor", "simt"])
def test_wide_shape_matches_oracle(bflib, oracle, kernel):
    d = bflib.Dims(256, 2, D, 2, B)
    E = np.empty(d.esize, np.uint8)
    bflib.fill_random_host(E, 4, 0)
    A, G = _weights(bflib, 2, 4)
    want = oracle.form_beams(oracle.Dims(256, 2, D, 2, B), E, A, G)
    J = np.zeros(d.jsize, np.uint8)
    bflib.set_kernel(kernel)
    try:
        bflib.form_beams_ex(d, J, E, A, G)
        assert bflib.last_kernel() == kernel
    finally:
        bflib.set_kernel("auto")
    np.testing.assert_array_equal(J, want)


def test_server_weight_refresh_without_drain(bflib, cuda, oracle):
    F, T = 2, 256
    A0, G = _weights(bflib, F, 4)
    W = bflib.ResidentWeights(F, B, D, A0, G)
    srv = bflib.Server(W, max_batch=8, max_inflight=2)
    versions = [A0]
    chunks = []
    for i in range(20):
        if i and i % 4 == 0:  # refresh from seed 4 + k, chunks still in flight
            A, _ = _weights(bflib, F, 4 + len(versions))
            srv.update_weights(A, G)
            versions.append(A)
        c = i % F
        E = np.empty(T * D * 2, np.uint8)
        bflib.fill_random_host(E, 500 + i, 0)
        J = np.zeros(B * 2 * T, np.uint8)
        chunks.append((c, E, J, len(versions) - 1, srv.submit(c, T, E, J)))
    for *_, t in chunks:
        srv.wait(t)
    st = srv.stats()
    srv.close()
    W.close()
    assert st["weight_updates"] == len(versions) - 1 == 4
    for c, E, J, v, _ in chunks:
        A = versions[v]
        want = oracle.form_beams(oracle.Dims(T, 1, D, 2, B), E, A[c * B * D:(c + 1) * B * D], G[c * B:(c + 1) * B])
        np.testing.assert_array_equal(J, want, err_msg=f"channel {c} version {v}")


def test_server_keeps_caller_weights(bflib, cuda):
    """A refresh never writes the caller's resident weights."""
    F, T = 1, 64
    A0, G = _weights(bflib, F, 9)
    W = bflib.ResidentWeights(F, B, D, A0, G)
    E = np.empty(T * D * 2, np.uint8)
    bflib.fill_random_host(E, 1, 0)
    Ed = cuda.from_numpy(E).cuda()
    J0 = cuda.empty((B * 2 * T,), dtype=cuda.uint8, device="cuda")
    W.form_beams(J0, Ed, T)
    bflib.stream_status()
    srv = bflib.Server(W)
    for k in range(5):  # more refreshes than versions: slots are reused
        A, _ = _weights(bflib, F, 20 + k)
        srv.update_weights(A, G)
    srv.close()
    J1 = cuda.empty_like(J0)
    W.form_beams(J1, Ed, T)
    bflib.stream_status()
    assert cuda.equal(J0, J1)


def test_tensor_peak_is_measured(bflib):
    tf = bflib.tensor_peak_tflops()
    assert 500.0 < tf < 20000.0


def test_dp4a_peak_is_measured(bflib):
    rate = bflib.dp4a_peak_per_s()
    assert 1e12 < rate < 1e15


def test_server_refresh_under_load(bflib, cuda):
    """Refreshes while several grouped launches are in flight (each chunk
    checked against a plain launch with the weights of its submission).  This
    load once exposed a missing cross-proxy fence between the unpack's reads
    of a raw E slot and the next TMA write into it."""
    F, T, nver, per = 16, 4096, 9, 4
    d = bflib.Dims(T, F, D, 2, B)
    G = cuda.from_numpy(bflib.gains(d)).cuda()
    As = []
    for k in range(nver):
        A = cuda.empty(d.asize, dtype=cuda.uint8, device="cuda")
        bflib.fill_random_device(A, 40 + k, 1)
        As.append(A)
    Es = []
    for i in range(4):
        E = cuda.empty(d.esize, dtype=cuda.uint8, device="cuda")
        bflib.fill_random_device(E, 60 + i, 0)
        Es.append(E)
    ref = bflib.ResidentWeights(F, B, D, As[0], G)
    Jt = cuda.empty(d.jsize, dtype=cuda.uint8, device="cuda")
    want = {}
    for k in range(nver):
        ref.update(As[k], G)
        for i in range(4):
            ref.form_beams(Jt, Es[i], T)
            bflib.stream_status()
            want[(k, i)] = bflib.adler32_device(Jt)
    ref.close()
    W = bflib.ResidentWeights(F, B, D, As[0], G)
    cuda.cuda.synchronize()
    bad = 0
    for rep in range(3):
        srv = bflib.Server(W, hbm_budget_bytes=1 << 30, max_batch=64, max_inflight=3, spin_wait=True)
        Js = [cuda.empty(d.jsize, dtype=cuda.uint8, device="cuda") for _ in range(per * nver)]
        subs, v = [], 0
        for i in range(per * nver):
            if i and i % per == 0:
                v += 1
                srv.update_weights(As[v], G)
            subs.append((srv.submit(0, T, Es[i % 4], Js[i], nchannels=F), v, i % 4, i))
        srv.drain()
        for t, *_ in subs:
            srv.wait(t)
        srv.close()
        bad += sum(bflib.adler32_device(Js[j]) != want[(v, i)] for _, v, i, j in subs)
    W.close()
    assert bad == 0
