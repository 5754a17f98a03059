"""TEST INFRASTRUCTURE ONLY: runs the reference's own exact GPU kernel.

`oracle/build_ref.sh` compiles the reference's `cuda.cu` (the wmma s4 kernel
`form_beams`, cuda.cu:35-253), unmodified, as device code for sm_103a into
oracle/_ref/<T>_<F>_<D>_<P>_<B>/cuda.cubin, with the kernel's entry name beside
it.  This module loads that cubin through the CUDA driver API into the calling
thread's current context (the one PyTorch made current) and launches it the
way the reference's main does (cuda.cu:290-296): one block per frequency,
4 x 8 x 12 threads, no dynamic shared memory.  The launch covers every beam
only when nbeams / 8 is a multiple of 12 (cuda.cu:76), which `available`
checks before anything runs.

Only the tests and the benchmark's reference arm use it, as a second
reference next to the CPU oracle; nothing of the product path loads it.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
_REF_DIR = os.path.join(_HERE, "_ref")
_BLOCK = (4, 8, 12)  # cuda.cu:295


def shape_dir(ntimes: int, nfrequencies: int, ndishes: int, npolarizations: int, nbeams: int) -> str:
    return os.path.join(_REF_DIR, f"{ntimes}_{nfrequencies}_{ndishes}_{npolarizations}_{nbeams}")


def available(ntimes: int, nfrequencies: int, ndishes: int, npolarizations: int, nbeams: int) -> bool:
    """True when the cubin for this shape was built and the reference's launch
    covers the shape exactly (cuda.cu:63-76)."""
    if nbeams % 8 or (nbeams // 8) % _BLOCK[2] or ndishes % 32 or ntimes % 8 or npolarizations != 2:
        return False
    d = shape_dir(ntimes, nfrequencies, ndishes, npolarizations, nbeams)
    return os.path.exists(os.path.join(d, "cuda.cubin")) and os.path.exists(os.path.join(d, "cuda.entry"))


class _Driver:
    def __init__(self):
        self.lib = ctypes.CDLL("libcuda.so.1")
        for name, args in (
            ("cuInit", [ctypes.c_uint]),
            ("cuCtxGetCurrent", [ctypes.POINTER(ctypes.c_void_p)]),
            ("cuModuleLoad", [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]),
            ("cuModuleGetFunction", [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p, ctypes.c_char_p]),
            ("cuModuleUnload", [ctypes.c_void_p]),
            ("cuLaunchKernel", [ctypes.c_void_p] + [ctypes.c_uint] * 7 + [ctypes.c_void_p,
                                                                        ctypes.POINTER(ctypes.c_void_p),
                                                                        ctypes.c_void_p]),
        ):
            fn = getattr(self.lib, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int

    def check(self, rc: int, what: str) -> None:
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")


class ReferenceKernel:
    """The reference's `form_beams` kernel for one compiled shape."""

    def __init__(self, ntimes: int, nfrequencies: int, ndishes: int, npolarizations: int, nbeams: int):
        if not available(ntimes, nfrequencies, ndishes, npolarizations, nbeams):
            raise FileNotFoundError("the reference GPU kernel is not built for this shape")
        d = shape_dir(ntimes, nfrequencies, ndishes, npolarizations, nbeams)
        with open(os.path.join(d, "cuda.entry")) as f:
            entry = f.read().strip()
        self.nfrequencies = nfrequencies
        self._drv = _Driver()
        self._drv.check(self._drv.lib.cuInit(0), "cuInit")
        ctx = ctypes.c_void_p()
        self._drv.check(self._drv.lib.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context on this thread (initialise the device first)")
        self._mod = ctypes.c_void_p()
        self._drv.check(self._drv.lib.cuModuleLoad(ctypes.byref(self._mod), os.path.join(d, "cuda.cubin").encode()),
                        "cuModuleLoad")
        self._fn = ctypes.c_void_p()
        self._drv.check(self._drv.lib.cuModuleGetFunction(ctypes.byref(self._fn), self._mod, entry.encode()),
                        "cuModuleGetFunction")

    def launch(self, J: int, E: int, A: int, G: int, stream: int = 0) -> None:
        """One launch on device pointers J, E, A, G (cuda.cu:35-36) in `stream`."""
        vals = [ctypes.c_uint64(J), ctypes.c_uint64(E), ctypes.c_uint64(A), ctypes.c_uint64(G)]
        params = (ctypes.c_void_p * 4)(*[ctypes.cast(ctypes.byref(v), ctypes.c_void_p) for v in vals])
        self._drv.check(
            self._drv.lib.cuLaunchKernel(self._fn, self.nfrequencies, 1, 1, *_BLOCK, 0, ctypes.c_void_p(stream),
                                         params, None),
            "cuLaunchKernel")

    def close(self) -> None:
        if getattr(self, "_mod", None) and self._mod.value:
            self._drv.lib.cuModuleUnload(self._mod)
            self._mod = ctypes.c_void_p()
