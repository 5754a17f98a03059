"""Batched uneven problems in one persistent launch: every problem's J equals
the oracle's and the per-problem launch's, alone and in the mix."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(bf, torch, T, F, D, B, seed):
    d = bf.Dims(T, F, D, 2, B)
    E = np.empty(d.esize, np.uint8)
    A = np.empty(d.asize, np.uint8)
    bf.fill_random_host(E, seed, 0)
    bf.fill_random_host(A, seed, 1)
    G = bf.gains(d)
    W = bf.ResidentWeights(F, B, D, A, G)
    Ed = torch.from_numpy(E).cuda()
    Jd = torch.full((d.jsize,), 0x5A, dtype=torch.uint8, device="cuda")
    return d, (E, A, G), W, Ed, Jd


def _oracle(oracle, d, E, A, G):
    return oracle.form_beams(oracle.Dims(d.ntimes, d.nfrequencies, d.ndishes, 2, d.nbeams), E, A, G)


def _check_layout(L):
    """A launch's layout follows its widest pass: at most 16 beams two CTAs per
    SM (two TMEM stages each); at most 64 four or more stages and two unpack
    groups; wider one group beside fewer than four stages."""
    if L["max_nb_pass"] <= 16:
        assert (L["ctas_per_sm"], L["unpack_groups"], L["stages"]) == (2, 1, 2), L
    elif L["max_nb_pass"] <= 64:
        assert L["ctas_per_sm"] == 1 and L["unpack_groups"] == 2 and L["stages"] >= 4, L
    else:
        assert L["ctas_per_sm"] == 1 and L["unpack_groups"] == 1 and L["stages"] < 4, L


def test_batch_uneven_shapes(bflib, cuda, oracle):
    rng = np.random.default_rng(2)
    shapes = []
    for i in range(12):
        T = int(rng.choice([16, 48, 64, 208, 512, 1024, 1296]))
        B = int(rng.choice([8, 16, 40, 64, 96, 128, 200]))
        F = int(rng.choice([1, 1, 2]))
        shapes.append((T, F, 512, B))
    probs = [_problem(bflib, cuda, T, F, D, B, 100 + i) for i, (T, F, D, B) in enumerate(shapes)]
    batch = bflib.Batch([(W, d.ntimes, Ed, Jd) for d, _, W, Ed, Jd in probs])
    info = batch.info()
    assert info["ntiles"] > 0
    batch.run()
    bflib.stream_status()
    for d, (E, A, G), W, Ed, Jd in probs:
        np.testing.assert_array_equal(Jd.cpu().numpy(), _oracle(oracle, d, E, A, G), err_msg=str(d))
    # the same problem alone through the per-problem launch gives the same bytes
    d, (E, A, G), W, Ed, Jd = probs[3]
    J1 = cuda.empty_like(Jd)
    W.form_beams(J1, Ed, d.ntimes)
    bflib.stream_status()
    assert cuda.equal(J1, Jd)
    batch.close()


def test_batch_replay_sees_new_inputs(bflib, cuda, oracle):
    """The captured graph reads the problems' buffers on every run."""
    probs = [_problem(bflib, cuda, T, 1, 512, B, 7 + T) for T, B in [(256, 96), (64, 16), (512, 128)]]
    batch = bflib.Batch([(W, d.ntimes, Ed, Jd) for d, _, W, Ed, Jd in probs])
    for rep in range(2):
        for k, (d, (E, A, G), W, Ed, Jd) in enumerate(probs):
            E2 = np.empty_like(E)
            bflib.fill_random_host(E2, 1000 + 10 * rep + k, 0)
            Ed.copy_(cuda.from_numpy(E2))
            probs[k] = (d, (E2, A, G), W, Ed, Jd)
        batch.run()
        bflib.stream_status()
        for d, (E, A, G), W, Ed, Jd in probs:
            np.testing.assert_array_equal(Jd.cpu().numpy(), _oracle(oracle, d, E, A, G))
    batch.close()


def test_batch_narrow_passes_two_groups(bflib, cuda, oracle):
    """Only passes of at most 64 beams (b = 16, 40, 64, and 128 as two passes of
    64): the 40- and 64-beam passes run four or more unpacked stages and two
    unpack groups, the 8- and 16-beam ones the same or, in a launch of their
    own, two CTAs per SM; every problem equals the oracle."""
    shapes = [(512, 1, 512, 16), (208, 2, 512, 40), (1024, 1, 512, 64), (256, 2, 512, 128), (64, 1, 512, 8)]
    probs = [_problem(bflib, cuda, T, F, D, B, 300 + i) for i, (T, F, D, B) in enumerate(shapes)]
    batch = bflib.Batch([(W, d.ntimes, Ed, Jd) for d, _, W, Ed, Jd in probs])
    launches = batch.info()["launches"]
    assert 1 <= len(launches) <= 2 and launches[0]["max_nb_pass"] == 64
    for L in launches:
        _check_layout(L)
    batch.run()
    bflib.stream_status()
    for d, (E, A, G), W, Ed, Jd in probs:
        np.testing.assert_array_equal(Jd.cpu().numpy(), _oracle(oracle, d, E, A, G), err_msg=str(d))
    batch.close()


def test_batch_narrowest_passes_two_ctas_per_sm(bflib, cuda, oracle):
    """Only passes of at most 16 beams (b = 8, 12, 16, ragged t): one launch of
    two CTAs per SM; every problem equals the oracle."""
    shapes = [(4096, 2, 512, 16), (208, 1, 512, 8), (1296, 3, 512, 12), (64, 1, 512, 16), (2048, 1, 512, 16)]
    probs = [_problem(bflib, cuda, T, F, D, B, 400 + i) for i, (T, F, D, B) in enumerate(shapes)]
    batch = bflib.Batch([(W, d.ntimes, Ed, Jd) for d, _, W, Ed, Jd in probs])
    (L,) = batch.info()["launches"]
    assert L["max_nb_pass"] == 16 and L["problems"] == len(shapes)
    _check_layout(L)
    batch.run()
    bflib.stream_status()
    for d, (E, A, G), W, Ed, Jd in probs:
        np.testing.assert_array_equal(Jd.cpu().numpy(), _oracle(oracle, d, E, A, G), err_msg=str(d))
    batch.close()


def test_batch_rejects_mixed_dishes_and_odd_times(bflib, cuda):
    a = _problem(bflib, cuda, 64, 1, 512, 16, 1)
    b = _problem(bflib, cuda, 64, 1, 256, 16, 2)
    with pytest.raises(bflib.BeamformError) as ei:
        bflib.Batch([(x[2], x[0].ntimes, x[3], x[4]) for x in (a, b)])
    assert ei.value.status == bflib.ERR_UNSUPPORTED
    c = _problem(bflib, cuda, 40, 1, 512, 16, 3)
    with pytest.raises(bflib.BeamformError):
        bflib.Batch([(c[2], 40, c[3], c[4])])


def test_batched_workload_all_problems(bflib, cuda, oracle):
    """The batched workload itself (128 problems, f=1 d=512, t log-uniform in
    [512, 32768], b in {16..128}, seed 2) in one persistent launch: every
    problem's J equals the oracle's on the same seeded inputs."""
    import bench

    probs = []
    for i, (T, F, D, B) in enumerate(bench.batched_problems()):
        d = bflib.Dims(T, F, D, 2, B)
        E = cuda.empty(d.esize, dtype=cuda.uint8, device="cuda")
        A = cuda.empty(d.asize, dtype=cuda.uint8, device="cuda")
        bflib.fill_random_device(E, 2, 2 + 2 * i)
        bflib.fill_random_device(A, 2, 3 + 2 * i)
        W = bflib.ResidentWeights(F, B, D, A, cuda.from_numpy(bflib.gains(d)).cuda())
        J = cuda.full((d.jsize,), 0x5A, dtype=cuda.uint8, device="cuda")
        probs.append((d, W, E, J))
    batch = bflib.Batch([(W, d.ntimes, E, J) for d, W, E, J in probs])
    info = batch.info()
    launches = info["launches"]
    assert 1 <= len(launches) <= 3 and sum(L["problems"] for L in launches) == len(probs)
    assert sum(L["tiles"] for L in launches) == info["ntiles"]
    for L in launches:
        _check_layout(L)
    batch.run()
    bflib.stream_status()
    assert bench.batched_oracle_check(probs) == len(probs)
    batch.close()
    for _, W, _, _ in probs:
        W.close()
