"""The served stream: chunks submitted to the continuous-batching server come
back bit-exact (against the oracle and against a per-chunk resident launch),
whatever batch they were packed into, with host or device buffers, under a
small HBM budget that forces admission to wait for completions."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

F, B, D = 6, 96, 512


@pytest.fixture(scope="module")
def weights(bflib):
    d = bflib.Dims(16, F, D, 2, B)
    A = np.empty(d.asize, np.uint8)
    bflib.fill_random_host(A, 31, 1)
    G = bflib.gains(d)
    W = bflib.ResidentWeights(F, B, D, A, G)
    yield W, A, G
    W.close()


def _chunks(bflib, n, seed, sizes=(64, 256, 1024, 2048)):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nch = int(rng.choice([1, 1, 2]))
        c0 = int(rng.integers(0, F - nch + 1))
        T = int(rng.choice(sizes))
        E = np.empty(T * nch * D * 2, np.uint8)
        bflib.fill_random_host(E, 1000 * seed + i, 0)
        out.append((c0, nch, T, E))
    return out


def _expected(oracle, A, G, c0, nch, T, E):
    d = oracle.Dims(T, nch, D, 2, B)
    return oracle.form_beams(d, E, A[c0 * B * D:(c0 + nch) * B * D], G[c0 * B:(c0 + nch) * B])


@pytest.mark.parametrize("max_batch,max_inflight,spin", [(0, 0, False), (1, 1, False), (4, 2, True)])
def test_server_chunks_bit_exact(bflib, cuda, oracle, weights, max_batch, max_inflight, spin):
    W, A, G = weights
    chunks = _chunks(bflib, 24, 5)
    srv = bflib.Server(W, max_batch=max_batch, max_inflight=max_inflight, spin_wait=spin)
    tickets, outs = [], []
    for i, (c0, nch, T, E) in enumerate(chunks):
        on_device = i % 3 == 1
        Ein = cuda.from_numpy(E).cuda() if on_device else E
        J = (cuda.full((B * nch * 2 * T,), 0x5A, dtype=cuda.uint8, device="cuda") if i % 2
             else np.full(B * nch * 2 * T, 0x5A, np.uint8))
        tickets.append(srv.submit(c0, T, Ein, J, nchannels=nch))
        outs.append((Ein, J))
    lats = [srv.wait(t) for t in tickets]
    srv.drain()
    st = srv.stats()
    srv.close()
    assert all(x > 0 for x in lats)
    assert st["submitted"] == st["completed"] == len(chunks)
    if max_batch == 1:
        assert st["max_batch_seen"] == 1
    for (c0, nch, T, E), (_, J) in zip(chunks, outs):
        got = J.cpu().numpy() if hasattr(J, "cpu") else J
        np.testing.assert_array_equal(got, _expected(oracle, A, G, c0, nch, T, E), err_msg=f"{c0} {nch} {T}")


def test_server_matches_resident_launch(bflib, cuda, weights):
    """A chunk over all channels equals the resident single-problem launch."""
    W, A, G = weights
    T = 4096
    E = np.empty(T * F * D * 2, np.uint8)
    bflib.fill_random_host(E, 77, 0)
    Ed = cuda.from_numpy(E).cuda()
    J1 = cuda.empty((B * F * 2 * T,), dtype=cuda.uint8, device="cuda")
    W.form_beams(J1, Ed, T)
    bflib.stream_status()
    srv = bflib.Server(W)
    J2 = np.zeros(B * F * 2 * T, np.uint8)
    srv.wait(srv.submit(0, T, E, J2, nchannels=F))
    srv.close()
    np.testing.assert_array_equal(J1.cpu().numpy(), J2)


def test_server_small_budget_admission(bflib, cuda, oracle, weights):
    """A pool with room for only a few chunks: admission waits for completions,
    the pool never exceeds its budget, every chunk is still exact, and a chunk
    larger than the whole pool is refused at submission."""
    W, A, G = weights
    chunks = _chunks(bflib, 16, 9, sizes=(1024, 2048))
    per_chunk = 2048 * 2 * D * 2 + B * 2 * 2 * 2048
    budget = 3 * per_chunk
    srv = bflib.Server(W, hbm_budget_bytes=budget, max_batch=8, max_inflight=2)
    tickets, outs = [], []
    for c0, nch, T, E in chunks:
        J = np.zeros(B * nch * 2 * T, np.uint8)
        tickets.append(srv.submit(c0, T, E, J, nchannels=nch))
        outs.append(J)
    big_T = 16384
    with pytest.raises(bflib.BeamformError) as ei:
        srv.submit(0, big_T, np.zeros(big_T * 2 * D * 2, np.uint8), np.zeros(B * 2 * 2 * big_T, np.uint8),
                   nchannels=2)
    assert ei.value.status == bflib.ERR_OUT_OF_MEMORY
    for t in tickets:
        srv.wait(t)
    st = srv.stats()
    srv.close()
    assert st["pool_bytes"] == budget
    assert 0 < st["pool_peak_bytes"] <= budget
    assert st["completed"] == len(chunks)
    for (c0, nch, T, E), J in zip(chunks, outs):
        np.testing.assert_array_equal(J, _expected(oracle, A, G, c0, nch, T, E))


def test_server_rejects_bad_chunks(bflib, weights):
    W, A, G = weights
    srv = bflib.Server(W)
    E = np.zeros(40 * D * 2, np.uint8)
    J = np.zeros(B * 2 * 40, np.uint8)
    with pytest.raises(bflib.BeamformError) as ei:
        srv.submit(F, 16, E, J)  # channel out of range
    assert ei.value.status == bflib.ERR_INVALID_ARGUMENT
    with pytest.raises(bflib.BeamformError) as ei:
        srv.submit(0, 40, E, J)  # ntimes not a multiple of 16
    assert ei.value.status == bflib.ERR_UNSUPPORTED
    srv.close()


def _pinned_copy(cuda, a):
    p = cuda.empty(a.size, dtype=cuda.uint8, pin_memory=True).numpy()
    p[:] = a
    return p


@pytest.mark.parametrize("mode", ["pageable", "pinned", "no_ring"])
def test_server_pinned_staging_ring(bflib, cuda, oracle, weights, mode):
    """Pageable host buffers go through the server's pinned staging ring (E
    copied in at submit, J copied out on landing); pinned buffers and a server
    without a ring are copied directly.  All give the oracle's bytes."""
    W, A, G = weights
    chunks = _chunks(bflib, 12, 9)
    srv = bflib.Server(W, max_batch=4, max_inflight=2, staging_bytes=-1 if mode == "no_ring" else 0)
    tickets, outs = [], []
    for c0, nch, T, E in chunks:
        J = np.full(B * nch * 2 * T, 0x5A, np.uint8)
        if mode == "pinned":
            E, J = _pinned_copy(cuda, E), _pinned_copy(cuda, J)
        tickets.append(srv.submit(c0, T, E, J, nchannels=nch))
        outs.append(J)
    for t in tickets:
        srv.wait(t)
    st = srv.stats()
    srv.close()
    assert st["staged"] == (len(chunks) if mode == "pageable" else 0)
    for (c0, nch, T, E), J in zip(chunks, outs):
        np.testing.assert_array_equal(J, _expected(oracle, A, G, c0, nch, T, E), err_msg=f"{mode} {c0} {nch} {T}")


def test_server_small_staging_ring_back_pressure(bflib, oracle, weights):
    """A ring that holds about two chunks: one thread submitting many chunks
    without waiting blocks in submit until landed chunks free the ring, and
    every chunk still comes back right (no wait on the client is needed for
    the ring to drain)."""
    W, A, G = weights
    chunks = _chunks(bflib, 10, 11, sizes=(1024,))
    per_chunk = max(1024 * nch * D * 2 + B * nch * 2 * 1024 for _, nch, _, _ in chunks) + 512
    srv = bflib.Server(W, max_batch=2, max_inflight=2, staging_bytes=2 * per_chunk + 4096)
    tickets, outs = [], []
    for c0, nch, T, E in chunks:
        J = np.full(B * nch * 2 * T, 0x5A, np.uint8)
        tickets.append(srv.submit(c0, T, E, J, nchannels=nch))
        outs.append(J)
    srv.drain()
    for t in tickets:
        srv.wait(t)
    st = srv.stats()
    srv.close()
    assert st["staged"] == len(chunks)
    for (c0, nch, T, E), J in zip(chunks, outs):
        np.testing.assert_array_equal(J, _expected(oracle, A, G, c0, nch, T, E))


@pytest.mark.parametrize("max_batch,max_inflight,nslots,rate", [(0, 0, 5, 0.0), (1, 1, 5, 0.0), (0, 0, 64, 4000.0)])
def test_server_replay_native_load_generator(bflib, cuda, oracle, weights, max_batch, max_inflight, nslots, rate):
    """bf_server_replay submits on a schedule from native threads, reuses its
    J slots only after the previous chunk in the slot landed and was
    checksummed, and returns each landed J's adler32: every one equals the
    oracle's for its chunk (back to back with 5 slots, so submissions wait
    for slots; and a Poisson stream)."""
    import zlib

    import torch

    W, A, G = weights
    rng = np.random.default_rng(17)
    contents = []
    for k in range(6):
        c0 = int(rng.integers(0, F))
        T = int(rng.choice([64, 256, 1024]))
        E = torch.empty(T * D * 2, dtype=torch.uint8, pin_memory=True).numpy()
        bflib.fill_random_host(E, 500 + k, 0)
        contents.append((c0, T, E, zlib.adler32(_expected(oracle, A, G, c0, 1, T, E).tobytes())))
    n = 60
    picks = rng.integers(len(contents), size=n)
    arrivals = np.zeros(n) if rate == 0 else np.cumsum(rng.exponential(1.0 / rate, n))
    maxj = B * 2 * 1024
    ring = torch.empty(nslots * maxj, dtype=torch.uint8, pin_memory=True).numpy()
    slots = [ring[k * maxj:(k + 1) * maxj] for k in range(nslots)]
    srv = bflib.Server(W, max_batch=max_batch, max_inflight=max_inflight)
    r = srv.replay([contents[p][0] for p in picks], [contents[p][1] for p in picks], [contents[p][2] for p in picks],
                   slots, [B * 2 * contents[p][1] for p in picks], arrivals, check_threads=3)
    st = srv.stats()
    srv.close()
    assert [int(a) for a in r["adler32"]] == [contents[p][3] for p in picks]
    assert st["completed"] == n and (r["latency_s"] > 0).all() and r["wall_s"] > 0
    if nslots < n and rate == 0:
        assert r["slot_stalls"] > 0
