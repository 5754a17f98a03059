"""The alternative wire formats: A2 input (A2linear, dish order of
cuda4.cu:1468-1494) and J2 output (J2linear) give the reference's values --
J2 equals the oracle's J permuted, A2 gives the same J as A -- on both
kernels, through the device and the host-pointer (chunked) paths."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(256, 2, 512, 96), (128, 3, 256, 40), (192, 1, 512, 200), (320, 2, 512, 16)]


def _inputs(bflib, T, F, D, B, seed):
    d = bflib.Dims(T, F, D, 2, B)
    E = np.empty(d.esize, np.uint8)
    A = np.empty(d.asize, np.uint8)
    bflib.fill_random_host(E, seed, 0)
    bflib.fill_random_host(A, seed, 1)
    return d, E, A, bflib.gains(d)


@pytest.mark.parametrize("kernel", ["tensor", "simt", "simt4"])
@pytest.mark.parametrize("shape", SHAPES)
def test_layouts_match_oracle(bflib, oracle, kernel, shape):
    d, E, A, G = _inputs(bflib, *shape, seed=sum(shape))
    od = oracle.Dims(d.ntimes, d.nfrequencies, d.ndishes, 2, d.nbeams)
    J = oracle.form_beams(od, E, A, G)
    J2 = oracle.J_to_J2(od, J)
    A2 = oracle.A_to_A2(od, A)
    bflib.set_kernel(kernel)
    try:
        for a_name, a_arr in (("linear", A), ("a2", A2)):
            for j_name, want in (("linear", J), ("j2", J2)):
                out = np.zeros(d.jsize, np.uint8)
                bflib.form_beams_layout(d, out, E, a_arr, G, a_layout=a_name, j_layout=j_name)
                assert bflib.last_kernel() == kernel
                np.testing.assert_array_equal(out, want, err_msg=f"{a_name} {j_name}")
    finally:
        bflib.set_kernel("auto")


def test_layouts_device_pointers(bflib, cuda, oracle):
    d, E, A, G = _inputs(bflib, 512, 2, 512, 96, seed=11)
    od = oracle.Dims(d.ntimes, d.nfrequencies, d.ndishes, 2, d.nbeams)
    J2 = oracle.J_to_J2(od, oracle.form_beams(od, E, A, G))
    A2 = oracle.A_to_A2(od, A)
    Jd = cuda.zeros(d.jsize, dtype=cuda.uint8, device="cuda")
    bflib.form_beams_layout(d, Jd, cuda.from_numpy(E).cuda(), cuda.from_numpy(A2).cuda(), cuda.from_numpy(G).cuda(),
                            a_layout="a2", j_layout="j2")
    bflib.stream_status()
    np.testing.assert_array_equal(Jd.cpu().numpy(), J2)


def test_j2_through_the_chunked_host_path(bflib, oracle, monkeypatch):
    """The host-pointer path cuts E into time chunks; each chunk writes its
    rows of J2 in place."""
    monkeypatch.setenv("BF_HOST_CHUNK_BYTES", str(64 * 4 * 512 * 2))
    d, E, A, G = _inputs(bflib, 1024, 4, 512, 96, seed=12)
    od = oracle.Dims(d.ntimes, d.nfrequencies, d.ndishes, 2, d.nbeams)
    J2 = oracle.J_to_J2(od, oracle.form_beams(od, E, A, G))
    out = np.zeros(d.jsize, np.uint8)
    bflib.form_beams_layout(d, out, E, A, G, j_layout="j2")
    np.testing.assert_array_equal(out, J2)
