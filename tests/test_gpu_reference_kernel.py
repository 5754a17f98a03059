"""The reference's own exact GPU kernel (cuda.cu:35-253, compiled unmodified
for sm_103a into oracle/_ref/) against this library's tensor-core kernel and
the oracle, on the same seeded device inputs: all three J arrays are equal
byte for byte.  Skipped where the reference kernel was not built."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,seed", [((2048, 16, 512, 2, 96), 0)])
def test_reference_gpu_kernel_matches(bflib, cuda, oracle, shape, seed):
    from oracle import ref_gpu

    if not ref_gpu.available(*shape):
        pytest.skip("reference GPU kernel not built for this shape")
    d = bflib.Dims(*shape)
    E, A, G = bflib.seeded_host_inputs(d, seed)
    Ed, Ad, Gd = (cuda.from_numpy(x).cuda() for x in (E, A, G))
    Jr = cuda.full((d.jsize,), 0x5A, dtype=cuda.uint8, device="cuda")
    k = ref_gpu.ReferenceKernel(*shape)
    try:
        k.launch(Jr.data_ptr(), Ed.data_ptr(), Ad.data_ptr(), Gd.data_ptr(), cuda.cuda.current_stream().cuda_stream)
        cuda.cuda.synchronize()
    finally:
        k.close()
    Jt = cuda.full((d.jsize,), 0xA5, dtype=cuda.uint8, device="cuda")
    bflib.set_kernel("tensor")
    try:
        bflib.form_beams_ex(d, Jt, Ed, Ad, Gd)
        bflib.stream_status()
    finally:
        bflib.set_kernel("auto")
    assert cuda.equal(Jr, Jt)
    expect = oracle.form_beams(oracle.Dims(*shape), E, A, G)
    np.testing.assert_array_equal(Jr.cpu().numpy(), expect)
