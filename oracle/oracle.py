"""TEST INFRASTRUCTURE ONLY: ctypes wrapper around the CPU oracle (oracle.c).

The oracle restates the reference beamformer (eschnett/beamforming, cpu.cxx:15-46)
on the CPU.  It is the checker for the CUDA path; only the tests, the smoke
check and the benchmark's CPU-baseline leg import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle.so")
_lib = None


class _Dims(ctypes.Structure):
    _fields_ = [
        ("ntimes", ctypes.c_int64),
        ("nfrequencies", ctypes.c_int64),
        ("ndishes", ctypes.c_int64),
        ("npolarizations", ctypes.c_int64),
        ("nbeams", ctypes.c_int64),
    ]


@dataclass(frozen=True)
class Dims:
    """Problem shape; the reference's compile-time sizes (arraysizes.hxx:22-27)."""

    ntimes: int
    nfrequencies: int
    ndishes: int
    npolarizations: int = 2
    nbeams: int = 96

    @property
    def esize(self) -> int:  # bytes of E (Esize / 2, arraysizes.hxx:79)
        return self.ntimes * self.nfrequencies * self.ndishes * self.npolarizations

    @property
    def asize(self) -> int:  # bytes of A (Asize / 2, arraysizes.hxx:114)
        return self.nfrequencies * self.nbeams * self.ndishes

    @property
    def gsize(self) -> int:  # floats of G (Gsize, arraysizes.hxx:135)
        return self.nfrequencies * self.nbeams

    @property
    def jsize(self) -> int:  # bytes of J (Jsize / 2, arraysizes.hxx:91)
        return self.nbeams * self.nfrequencies * self.npolarizations * self.ntimes

    @property
    def cmacs(self) -> int:  # complex multiply-adds of one form_beams call
        return self.ntimes * self.nfrequencies * self.npolarizations * self.nbeams * self.ndishes

    def c(self) -> _Dims:
        return _Dims(self.ntimes, self.nfrequencies, self.ndishes, self.npolarizations, self.nbeams)


def build() -> str:
    """Compile liboracle.so with make (portable flags) and return its path."""
    subprocess.run(["make", "-s", "-C", _HERE, "liboracle.so"], check=True)
    return _LIB_PATH


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(
            os.path.join(_HERE, "oracle.c")
        ):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        L.bfo_encode.argtypes = [ctypes.c_int, ctypes.c_int]
        L.bfo_encode.restype = ctypes.c_uint8
        L.bfo_decode_re.argtypes = [ctypes.c_uint8]
        L.bfo_decode_re.restype = ctypes.c_int
        L.bfo_decode_im.argtypes = [ctypes.c_uint8]
        L.bfo_decode_im.restype = ctypes.c_int
        L.bfo_form_beams.argtypes = [ctypes.POINTER(_Dims), u8p, u8p, u8p, ctypes.POINTER(ctypes.c_float), ctypes.c_int]
        L.bfo_form_beams.restype = None
        L.bfo_raw_sum.argtypes = [ctypes.POINTER(_Dims), u8p, u8p] + [ctypes.c_int64] * 4 + [
            ctypes.POINTER(ctypes.c_int32)
        ] * 2
        L.bfo_raw_sum.restype = None
        L.bfo_J_to_J2.argtypes = [ctypes.POINTER(_Dims), u8p, u8p]
        L.bfo_J_to_J2.restype = None
        L.bfo_A_to_A2.argtypes = [ctypes.POINTER(_Dims), u8p, u8p]
        L.bfo_A_to_A2.restype = None
        L.bfo_adler32.argtypes = [u8p, ctypes.c_size_t]
        L.bfo_adler32.restype = ctypes.c_uint32
        L.bfo_setup_pattern.argtypes = [ctypes.POINTER(_Dims), u8p, u8p, ctypes.POINTER(ctypes.c_float)]
        L.bfo_setup_pattern.restype = None
        L.bfo_gains.argtypes = [ctypes.POINTER(_Dims), ctypes.POINTER(ctypes.c_float)]
        L.bfo_gains.restype = None
        L.bfo_fill_random.argtypes = [u8p, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_uint64]
        L.bfo_fill_random.restype = None
        _lib = L
    return _lib


def _u8(a: np.ndarray):
    assert a.dtype == np.uint8 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))


def _f32(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def encode(re: int, im: int) -> int:
    return int(lib().bfo_encode(re, im))


def decode(data: int) -> tuple[int, int]:
    return int(lib().bfo_decode_re(data)), int(lib().bfo_decode_im(data))


def form_beams(dims: Dims, E: np.ndarray, A: np.ndarray, G: np.ndarray, nthreads: int = 0) -> np.ndarray:
    """J[b][f][p][t] bytes from E, A, G (cpu.cxx:15-46)."""
    assert E.size == dims.esize and A.size == dims.asize and G.size == dims.gsize
    J = np.empty(dims.jsize, dtype=np.uint8)
    d = dims.c()
    lib().bfo_form_beams(ctypes.byref(d), _u8(J), _u8(E), _u8(A), _f32(G), nthreads)
    return J


def raw_sum(dims: Dims, E: np.ndarray, A: np.ndarray, b: int, f: int, p: int, t: int) -> tuple[int, int]:
    re, im = ctypes.c_int32(), ctypes.c_int32()
    d = dims.c()
    lib().bfo_raw_sum(ctypes.byref(d), _u8(E), _u8(A), b, f, p, t, ctypes.byref(re), ctypes.byref(im))
    return re.value, im.value


def A_to_A2(dims: Dims, A: np.ndarray) -> np.ndarray:
    """A[f][b][d] -> A2[f][b][c][d'] (A2linear, arraysizes.hxx:125; cuda4.cu:1468-1494)."""
    if dims.ndishes not in (256, 512):
        raise ValueError("A2 is defined for ndishes 256 and 512")
    A2 = np.full_like(A, 0x88)
    d = dims.c()
    lib().bfo_A_to_A2(ctypes.byref(d), _u8(A2), _u8(A))
    return A2


def J_to_J2(dims: Dims, J: np.ndarray) -> np.ndarray:
    J2 = np.empty_like(J)
    d = dims.c()
    lib().bfo_J_to_J2(ctypes.byref(d), _u8(J2), _u8(J))
    return J2


def adler32(data: np.ndarray) -> int:
    data = np.ascontiguousarray(data).view(np.uint8).reshape(-1)
    return int(lib().bfo_adler32(_u8(data), data.size))


def setup_pattern(dims: Dims) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """The reference's deterministic inputs (arraysizes.cxx:8-52)."""
    E = np.empty(dims.esize, dtype=np.uint8)
    A = np.empty(dims.asize, dtype=np.uint8)
    G = np.empty(dims.gsize, dtype=np.float32)
    d = dims.c()
    lib().bfo_setup_pattern(ctypes.byref(d), _u8(E), _u8(A), _f32(G))
    return E, A, G


def gains(dims: Dims) -> np.ndarray:
    G = np.empty(dims.gsize, dtype=np.float32)
    d = dims.c()
    lib().bfo_gains(ctypes.byref(d), _f32(G))
    return G


def fill_random(n: int, seed: int, stream: int) -> np.ndarray:
    out = np.empty(n, dtype=np.uint8)
    lib().bfo_fill_random(_u8(out), n, seed, stream)
    return out


def seeded_inputs(dims: Dims, seed: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Seeded workload: E and A uniform bytes (each nibble uniform on [-8,7]),
    G from the reference's setup() formula at this shape."""
    return fill_random(dims.esize, seed, 0), fill_random(dims.asize, seed, 1), gains(dims)
