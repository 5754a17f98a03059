"""GB300-native CHORD beamformer: Python mirror of the C ABI in include/beamform.h.

The reference (eschnett/beamforming) exposes one operation,
``form_beams(J, E, A, G)`` (cpu.cxx:15-16), with sizes fixed at compile time
(arraysizes.hxx:22-27).  This package keeps that call -- ``form_beams(J, E, A, G)``
after ``set_dims(...)`` -- and adds the explicit, resident-weight, checksum and
workload-generator entry points of the C ABI.  All compute runs in
``libbeamform.so`` (CUDA, sm_103a); there is no CPU path.  Arrays are numpy
(host) or torch CUDA tensors (device), always uint8 bytes in the reference
layouts (float32 for G):

    E[t][f][d][p]   A[f][b][d]   G[f][b]   J[b][f][p][t]
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libbeamform.so")

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_UNSUPPORTED = 2
ERR_NO_DEVICE = 3
ERR_CUDA = 4
ERR_OUT_OF_MEMORY = 5
ERR_DEVICE_TIMEOUT = 6
ERR_NOT_CONFIGURED = 7
ERR_SIZE_MISMATCH = 8
ERR_TOO_LARGE = 9

PTR_HOST = 0
PTR_DEVICE = 1

KERNELS = {"auto": 0, "tensor": 1, "simt": 2, "simt4": 3}

# Every symbol the C header declares; the CPU tests check the library exports them.
EXPORTED_SYMBOLS = (
    "bf_set_dims",
    "bf_form_beams_adler",
    "form_beams",
    "bf_last_status",
    "bf_status_string",
    "bf_form_beams_ex",
    "bf_stream_status",
    "bf_set_kernel",
    "bf_plan_rings",
    "bf_set_test_stall",
    "bf_last_kernel",
    "bf_weights_create",
    "bf_weights_update",
    "bf_weights_destroy",
    "bf_form_beams_resident",
    "bf_form_beams_noalloc",
    "bf_batch_create",
    "bf_batch_run",
    "bf_batch_info",
    "bf_batch_shape",
    "bf_batch_destroy",
    "bf_tensor_peak",
    "bf_dp4a_peak",
    "bf_form_beams_layout",
    "bf_server_create",
    "bf_server_submit",
    "bf_server_update_weights",
    "bf_server_wait",
    "bf_server_drain",
    "bf_server_stats_get",
    "bf_server_replay",
    "bf_server_destroy",
    "bf_adler32_device",
    "bf_adler32_host",
    "bf_fill_random_device",
    "bf_fill_random_host",
    "bf_gains_host",
)


class BeamformError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = lib().bf_status_string(status).decode() if _lib is not None else f"status {status}"
        super().__init__(f"{what}: {msg} (status {status})" if what else f"{msg} (status {status})")


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
    """Problem shape: the reference's compile-time sizes (arraysizes.hxx:22-27)."""

    ntimes: int
    nfrequencies: int
    ndishes: int
    npolarizations: int = 2
    nbeams: int = 96

    @property
    def esize(self) -> int:
        return self.ntimes * self.nfrequencies * self.ndishes * self.npolarizations

    @property
    def asize(self) -> int:
        return self.nfrequencies * self.nbeams * self.ndishes

    @property
    def gsize(self) -> int:
        return self.nfrequencies * self.nbeams

    @property
    def jsize(self) -> int:
        return self.nbeams * self.nfrequencies * self.npolarizations * self.ntimes

    @property
    def cmacs(self) -> int:
        """Complex multiply-adds of one pass: t * f * p * b * d."""
        return self.ntimes * self.nfrequencies * self.npolarizations * self.nbeams * self.ndishes

    def c(self) -> _Dims:
        return _Dims(self.ntimes, self.nfrequencies, self.ndishes, self.npolarizations, self.nbeams)


_lib = None


def lib() -> ctypes.CDLL:
    """Loads libbeamform.so (built by ``beamforming_gb300.build.build()``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -m beamforming_gb300.build` "
                "(the beamformer has no CPU fallback)"
            )
        L = ctypes.CDLL(LIB_PATH)
        vp, u8p, fp = ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p
        D = ctypes.POINTER(_Dims)
        L.bf_set_dims.argtypes = [D]
        L.form_beams.argtypes = [u8p, u8p, u8p, fp]
        L.form_beams.restype = None
        L.bf_last_status.argtypes = []
        L.bf_status_string.argtypes = [ctypes.c_int]
        L.bf_status_string.restype = ctypes.c_char_p
        L.bf_form_beams_ex.argtypes = [D, u8p, u8p, u8p, fp, ctypes.c_int, vp]
        L.bf_form_beams_layout.argtypes = [D, u8p, u8p, u8p, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp]
        L.bf_form_beams_adler.argtypes = [D, u8p, u8p, u8p, fp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.POINTER(ctypes.c_uint32), vp]
        L.bf_stream_status.argtypes = [vp]
        L.bf_set_kernel.argtypes = [ctypes.c_int]
        L.bf_plan_rings.argtypes = [ctypes.c_int64, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_int)]
        L.bf_set_test_stall.argtypes = [ctypes.c_int]
        L.bf_last_kernel.argtypes = []
        L.bf_last_kernel.restype = ctypes.c_char_p
        L.bf_weights_create.argtypes = [
            ctypes.POINTER(vp),
            ctypes.c_int64,
            ctypes.c_int64,
            ctypes.c_int64,
            u8p,
            fp,
            ctypes.c_int,
            vp,
        ]
        L.bf_weights_update.argtypes = [vp, u8p, fp, ctypes.c_int, vp]
        L.bf_weights_destroy.argtypes = [vp]
        L.bf_form_beams_resident.argtypes = [vp, ctypes.c_int64, u8p, u8p, vp]
        L.bf_form_beams_noalloc.argtypes = [D, u8p, u8p, u8p, fp, vp]
        L.bf_batch_create.argtypes = [ctypes.POINTER(vp), ctypes.c_void_p, ctypes.c_int, vp]
        L.bf_batch_run.argtypes = [vp, vp]
        L.bf_batch_info.argtypes = [vp] + [ctypes.POINTER(ctypes.c_int)] * 4 + [ctypes.POINTER(ctypes.c_float)]
        L.bf_batch_shape.argtypes = [vp] + [ctypes.POINTER(ctypes.c_int)] * 7
        L.bf_batch_destroy.argtypes = [vp]
        L.bf_server_create.argtypes = [ctypes.POINTER(vp), vp, ctypes.POINTER(_ServerConfig)]
        L.bf_server_submit.argtypes = [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int64, u8p, ctypes.c_int, u8p,
                                       ctypes.c_int, ctypes.POINTER(ctypes.c_int64)]
        L.bf_tensor_peak.argtypes = [ctypes.POINTER(ctypes.c_double), vp]
        L.bf_dp4a_peak.argtypes = [ctypes.POINTER(ctypes.c_double), vp]
        L.bf_server_update_weights.argtypes = [vp, u8p, fp, ctypes.c_int]
        L.bf_server_wait.argtypes = [vp, ctypes.c_int64, ctypes.POINTER(ctypes.c_double)]
        L.bf_server_drain.argtypes = [vp]
        L.bf_server_stats_get.argtypes = [vp, ctypes.POINTER(_ServerStats)]
        dp = ctypes.POINTER(ctypes.c_double)
        L.bf_server_replay.argtypes = [vp, ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(vp), ctypes.c_int, ctypes.POINTER(vp), ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_int64), ctypes.c_int, dp, ctypes.c_int, dp, dp,
                                       ctypes.POINTER(ctypes.c_uint32), dp, ctypes.POINTER(ctypes.c_int64)]
        L.bf_adler32_host.argtypes = [u8p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint32)]
        L.bf_server_destroy.argtypes = [vp]
        L.bf_adler32_device.argtypes = [u8p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint32), vp]
        L.bf_fill_random_device.argtypes = [u8p, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_uint64, vp]
        L.bf_fill_random_host.argtypes = [u8p, ctypes.c_size_t, ctypes.c_uint64, ctypes.c_uint64]
        L.bf_gains_host.argtypes = [D, fp]
        for name in EXPORTED_SYMBOLS:
            if name not in ("form_beams", "bf_status_string", "bf_last_kernel"):
                getattr(L, name).restype = ctypes.c_int
        _lib = L
    return _lib


def _check(status: int, what: str) -> None:
    if status != OK:
        raise BeamformError(status, what)


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _ptr(x, dtype, nbytes_min: int, writable: bool = False) -> tuple[int, int]:
    """(address, ptr_kind) of a C-contiguous numpy array or CUDA tensor."""
    if _is_torch(x):
        import torch

        if not x.is_cuda:
            raise ValueError("torch tensors must be on a CUDA device; pass numpy arrays for host data")
        want = {np.uint8: torch.uint8, np.float32: torch.float32}[dtype]
        if x.dtype != want or not x.is_contiguous():
            raise ValueError(f"expected a contiguous {want} tensor")
        if x.numel() * x.element_size() < nbytes_min:
            raise ValueError("tensor too small for the shape")
        return x.data_ptr(), PTR_DEVICE
    if not isinstance(x, np.ndarray) or x.dtype != dtype or not x.flags["C_CONTIGUOUS"]:
        raise ValueError(f"expected a C-contiguous numpy {np.dtype(dtype)} array or a CUDA tensor")
    if writable and not x.flags["WRITEABLE"]:
        raise ValueError("output array is read-only")
    if x.nbytes < nbytes_min:
        raise ValueError("array too small for the shape")
    return x.ctypes.data, PTR_HOST


def _stream_handle(stream) -> int | None:
    if stream is None:
        try:
            import torch

            if torch.cuda.is_available() and torch.cuda.is_initialized():
                return torch.cuda.current_stream().cuda_stream
        except Exception:
            pass
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


# ------------------------------------------------------------------ drop-in


def set_dims(dims: Dims) -> None:
    """Sets the sizes form_beams() uses (the reference's arraysizes.hxx:22-27)."""
    d = dims.c()
    _check(lib().bf_set_dims(ctypes.byref(d)), "bf_set_dims")


def form_beams(J: np.ndarray, E: np.ndarray, A: np.ndarray, G: np.ndarray) -> None:
    """The reference call form_beams(J, E, A, G) (cpu.cxx:15-16) on host arrays,
    with sizes from set_dims().  Fills J in place; raises on failure."""
    for x, dt in ((J, np.uint8), (E, np.uint8), (A, np.uint8), (G, np.float32)):
        if not isinstance(x, np.ndarray) or x.dtype != dt or not x.flags["C_CONTIGUOUS"]:
            raise ValueError("form_beams takes C-contiguous host arrays (uint8 J, E, A; float32 G)")
    L = lib()
    L.form_beams(J.ctypes.data, E.ctypes.data, A.ctypes.data, G.ctypes.data)
    _check(L.bf_last_status(), "form_beams")


# -------------------------------------------------------------- explicit API


def form_beams_ex(dims: Dims, J, E, A, G, stream=None) -> None:
    """One pass with explicit sizes.  All-host arguments run synchronously;
    all-device (CUDA tensor) arguments are asynchronous on `stream`."""
    pj, kj = _ptr(J, np.uint8, dims.jsize, writable=True)
    pe, ke = _ptr(E, np.uint8, dims.esize)
    pa, ka = _ptr(A, np.uint8, dims.asize)
    pg, kg = _ptr(G, np.float32, 4 * dims.gsize)
    if len({kj, ke, ka, kg}) != 1:
        raise ValueError("E, A, G and J must all be host arrays or all CUDA tensors")
    d = dims.c()
    _check(
        lib().bf_form_beams_ex(ctypes.byref(d), pj, pe, pa, pg, kj, _stream_handle(stream) if kj else None),
        "bf_form_beams_ex",
    )


A_LAYOUTS = {"linear": 0, "a2": 1}
J_LAYOUTS = {"linear": 0, "j2": 1}


def form_beams_layout(dims: Dims, J, E, A, G, a_layout: str = "linear", j_layout: str = "linear",
                      stream=None) -> None:
    """form_beams_ex with A given in `a_layout` ("linear": A[f][b][d]; "a2":
    A2[f][b][c][d'], ndishes 256 or 512) and J written in `j_layout`
    ("linear": J[b][f][p][t]; "j2": J2[b][f][t][p])."""
    pj, kj = _ptr(J, np.uint8, dims.jsize, writable=True)
    pe, ke = _ptr(E, np.uint8, dims.esize)
    pa, ka = _ptr(A, np.uint8, dims.asize)
    pg, kg = _ptr(G, np.float32, 4 * dims.gsize)
    if len({kj, ke, ka, kg}) != 1:
        raise ValueError("E, A, G and J must all be host arrays or all CUDA tensors")
    d = dims.c()
    _check(
        lib().bf_form_beams_layout(ctypes.byref(d), pj, pe, pa, pg, A_LAYOUTS[a_layout], J_LAYOUTS[j_layout], kj,
                                   _stream_handle(stream) if kj else None),
        "bf_form_beams_layout",
    )


def form_beams_adler(dims: Dims, J, E, A, G, a_layout: str = "linear", j_layout: str = "linear",
                     stream=None) -> int:
    """form_beams_layout that also returns the adler32 of the whole J it wrote
    (the checksum the reference prints after form_beams), summed inside the
    tensor-core kernel instead of a second pass over J.  Synchronous."""
    pj, kj = _ptr(J, np.uint8, dims.jsize, writable=True)
    pe, ke = _ptr(E, np.uint8, dims.esize)
    pa, ka = _ptr(A, np.uint8, dims.asize)
    pg, kg = _ptr(G, np.float32, 4 * dims.gsize)
    if len({kj, ke, ka, kg}) != 1:
        raise ValueError("E, A, G and J must all be host arrays or all CUDA tensors")
    d = dims.c()
    out = ctypes.c_uint32(0)
    _check(
        lib().bf_form_beams_adler(ctypes.byref(d), pj, pe, pa, pg, A_LAYOUTS[a_layout], J_LAYOUTS[j_layout], kj,
                                  ctypes.byref(out), _stream_handle(stream) if kj else None),
        "bf_form_beams_adler",
    )
    return int(out.value)


def stream_status(stream=None) -> None:
    """Synchronizes the stream and raises if a kernel reported an error."""
    _check(lib().bf_stream_status(_stream_handle(stream)), "bf_stream_status")


def plan_rings(ndishes: int, max_nb_pass: int, wslots: int = 0, raw: int = 0) -> dict | None:
    """The ring layout the tensor-core kernel plans (host only, no GPU), or
    None where no layout fits: TMEM stages, W slots, raw E slots, unpack
    groups, CTAs per SM, K stages per tile, and the resources: shared memory
    bytes per CTA and the tensor-memory columns (allocated, per accumulator,
    the second accumulator's first column, stages per accumulator and the end
    of the stages' columns)."""
    out = (ctypes.c_int * 12)()
    if lib().bf_plan_rings(ndishes, max_nb_pass, wslots, raw, out) != 0:
        return None
    return dict(zip(("stages", "wslots", "raw", "groups", "ctas_per_sm", "nk", "smem_bytes", "tmem_cols",
                     "acc_cols", "acc2_col", "stages_per_acc", "stage_end_col"), list(out)))


def set_kernel(kind: str) -> None:
    _check(lib().bf_set_kernel(KERNELS[kind]), "bf_set_kernel")


def set_test_stall(on: bool) -> None:
    """Failure-path test hook: tensor-core launches issue no copies while on,
    so their bounded waits expire and the call raises ERR_DEVICE_TIMEOUT."""
    _check(lib().bf_set_test_stall(1 if on else 0), "bf_set_test_stall")


def last_kernel() -> str:
    return lib().bf_last_kernel().decode()


class ResidentWeights:
    """Beam weights A and gains G kept on the device in the tensor-core
    operand format; ``update`` refreshes them in place."""

    def __init__(self, nfrequencies: int, nbeams: int, ndishes: int, A, G, stream=None):
        self.nfrequencies, self.nbeams, self.ndishes = nfrequencies, nbeams, ndishes
        pa, ka = _ptr(A, np.uint8, nfrequencies * nbeams * ndishes)
        pg, kg = _ptr(G, np.float32, 4 * nfrequencies * nbeams)
        if ka != kg:
            raise ValueError("A and G must both be host arrays or both CUDA tensors")
        h = ctypes.c_void_p()
        _check(
            lib().bf_weights_create(
                ctypes.byref(h), nfrequencies, nbeams, ndishes, pa, pg, ka, _stream_handle(stream) if ka else None
            ),
            "bf_weights_create",
        )
        self._h = h

    def update(self, A, G, stream=None) -> None:
        pa, ka = _ptr(A, np.uint8, self.nfrequencies * self.nbeams * self.ndishes)
        pg, kg = _ptr(G, np.float32, 4 * self.nfrequencies * self.nbeams)
        if ka != kg:
            raise ValueError("A and G must both be host arrays or both CUDA tensors")
        _check(lib().bf_weights_update(self._h, pa, pg, ka, _stream_handle(stream) if ka else None), "bf_weights_update")

    def form_beams(self, J, E, ntimes: int, stream=None) -> None:
        """Asynchronous pass over device E (ntimes samples) into device J."""
        esz = ntimes * self.nfrequencies * self.ndishes * 2
        jsz = self.nbeams * self.nfrequencies * 2 * ntimes
        pj, kj = _ptr(J, np.uint8, jsz, writable=True)
        pe, ke = _ptr(E, np.uint8, esz)
        if kj != PTR_DEVICE or ke != PTR_DEVICE:
            raise ValueError("resident beamforming takes CUDA tensors")
        _check(
            lib().bf_form_beams_resident(self._h, ntimes, pj, pe, _stream_handle(stream)), "bf_form_beams_resident"
        )

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().bf_weights_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_int64), ("max_batch", ctypes.c_int), ("max_inflight", ctypes.c_int),
                ("spin_wait", ctypes.c_int), ("staging_bytes", ctypes.c_int64)]


class _ServerStats(ctypes.Structure):
    _fields_ = [
        (n, ctypes.c_int64)
        for n in ("submitted", "completed", "batches", "chunks_launched", "max_batch_seen", "pool_bytes",
                  "pool_peak_bytes", "weight_updates", "staged")
    ]


class Server:
    """Continuous-batching server over resident weights: ``submit`` chunks as
    they arrive, ``wait`` for a ticket (latency in seconds), ``drain``.  The
    server reads E and writes J after ``submit`` returns; the wrapper keeps
    the buffers referenced until the ticket is waited for.  Pageable host
    buffers go through the server's pinned staging ring (``staging_bytes``;
    0: 256 MiB, negative: none), pinned ones are copied directly."""

    def __init__(self, weights: "ResidentWeights", hbm_budget_bytes: int = 0, max_batch: int = 0,
                 max_inflight: int = 0, spin_wait: bool = False, staging_bytes: int = 0):
        self.weights = weights
        cfg = _ServerConfig(hbm_budget_bytes, max_batch, max_inflight, int(spin_wait), staging_bytes)
        h = ctypes.c_void_p()
        _check(lib().bf_server_create(ctypes.byref(h), weights._h, ctypes.byref(cfg)), "bf_server_create")
        self._h = h
        self._live: dict[int, tuple] = {}
        self._replay_keep: list = []  # buffers of a failed replay, held until close()

    def submit(self, channel: int, ntimes: int, E, J, nchannels: int = 1) -> int:
        w = self.weights
        pe, ke = _ptr(E, np.uint8, ntimes * nchannels * w.ndishes * 2)
        pj, kj = _ptr(J, np.uint8, w.nbeams * nchannels * 2 * ntimes, writable=True)
        t = ctypes.c_int64()
        _check(lib().bf_server_submit(self._h, channel, nchannels, ntimes, pe, ke, pj, kj, ctypes.byref(t)),
               "bf_server_submit")
        self._live[t.value] = (E, J)
        return t.value

    def update_weights(self, A, G) -> None:
        """New weights for chunks submitted from now on (no drain)."""
        w = self.weights
        pa, ka = _ptr(A, np.uint8, w.nfrequencies * w.nbeams * w.ndishes)
        pg, kg = _ptr(G, np.float32, 4 * w.nfrequencies * w.nbeams)
        if ka != kg:
            raise ValueError("A and G must both be host arrays or both CUDA tensors")
        _check(lib().bf_server_update_weights(self._h, pa, pg, ka), "bf_server_update_weights")

    def wait(self, ticket: int) -> float:
        lat = ctypes.c_double()
        _check(lib().bf_server_wait(self._h, ticket, ctypes.byref(lat)), "bf_server_wait")
        self._live.pop(ticket, None)
        return lat.value

    def drain(self) -> None:
        _check(lib().bf_server_drain(self._h), "bf_server_drain")

    def replay(self, channels, ntimes, E_list, J_slots, j_bytes, arrivals, check_threads: int = 4) -> dict:
        """Native load generator (bf_server_replay): chunk i (channel
        ``channels[i]``, ``ntimes[i]`` samples, input ``E_list[i]``, pinned
        host numpy arrays or CUDA tensors) is submitted ``arrivals[i]`` seconds
        after the call into J slot ``J_slots[i % len(J_slots)]`` (host numpy
        views, ``j_bytes[i]`` bytes used); returns per-chunk latency and
        lateness (seconds) and the adler32 of each landed J, the wall time to
        the last completion and the number of slot waits."""
        n = len(arrivals)
        w = self.weights
        ch = (ctypes.c_int * n)(*[int(c) for c in channels])
        nt = (ctypes.c_int64 * n)(*[int(t) for t in ntimes])
        jb = (ctypes.c_int64 * n)(*[int(b) for b in j_bytes])
        arr = (ctypes.c_double * n)(*[float(a) for a in arrivals])
        eptr, ekind = [], None
        for e, t in zip(E_list, ntimes):
            p, k = _ptr(e, np.uint8, int(t) * w.ndishes * 2)
            eptr.append(int(p))
            ekind = k if ekind is None else ekind
            if k != ekind:
                raise ValueError("E inputs must all be host arrays or all CUDA tensors")
        jptr, jkind = [], None
        for js in J_slots:
            p, k = _ptr(js, np.uint8, js.nbytes if hasattr(js, "nbytes") else js.numel(), writable=True)
            jptr.append(int(p))
            jkind = k if jkind is None else jkind
        E_arr = (ctypes.c_void_p * n)(*eptr)
        J_arr = (ctypes.c_void_p * len(jptr))(*jptr)
        lat = np.zeros(n)
        late = np.zeros(n)
        adl = np.zeros(n, dtype=np.uint32)
        wall = ctypes.c_double()
        stalls = ctypes.c_int64()
        dp = ctypes.POINTER(ctypes.c_double)
        rc = lib().bf_server_replay(
            self._h, n, ch, nt, E_arr, ekind, J_arr, len(jptr), jb, jkind, arr, check_threads,
            lat.ctypes.data_as(dp), late.ctypes.data_as(dp), adl.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
            ctypes.byref(wall), ctypes.byref(stalls))
        if rc != 0:
            # chunks already submitted may still be landing: keep their buffers until close()
            self._replay_keep.append((list(E_list), list(J_slots)))
        _check(rc, "bf_server_replay")
        return {"latency_s": lat, "late_s": late, "adler32": adl, "wall_s": wall.value, "slot_stalls": stalls.value}

    def stats(self) -> dict:
        st = _ServerStats()
        _check(lib().bf_server_stats_get(self._h, ctypes.byref(st)), "bf_server_stats_get")
        return {n: getattr(st, n) for n, _ in _ServerStats._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().bf_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _Problem(ctypes.Structure):
    _fields_ = [
        ("weights", ctypes.c_void_p),
        ("ntimes", ctypes.c_int64),
        ("E", ctypes.c_void_p),
        ("J", ctypes.c_void_p),
    ]


class Batch:
    """Many uneven problems (resident weights, ntimes, device E, device J) run
    as one persistent launch; the schedule is autotuned at creation and the
    launch replayed from a CUDA graph by ``run()``."""

    def __init__(self, problems, stream=None):
        arr = (_Problem * len(problems))()
        self._keep = []
        for i, (weights, ntimes, E, J) in enumerate(problems):
            pe, ke = _ptr(E, np.uint8, ntimes * weights.nfrequencies * weights.ndishes * 2)
            pj, kj = _ptr(J, np.uint8, weights.nbeams * weights.nfrequencies * 2 * ntimes, writable=True)
            if ke != PTR_DEVICE or kj != PTR_DEVICE:
                raise ValueError("batch problems take CUDA tensors")
            arr[i] = _Problem(weights._h, ntimes, pe, pj)
            self._keep.append((weights, E, J))
        h = ctypes.c_void_p()
        _check(lib().bf_batch_create(ctypes.byref(h), arr, len(problems), _stream_handle(stream)), "bf_batch_create")
        self._h = h

    def run(self, stream=None) -> None:
        _check(lib().bf_batch_run(self._h, _stream_handle(stream)), "bf_batch_run")

    def info(self) -> dict:
        nt, order, ws, raw, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        _check(
            lib().bf_batch_info(self._h, ctypes.byref(nt), ctypes.byref(order), ctypes.byref(ws), ctypes.byref(raw),
                                ctypes.byref(ms)),
            "bf_batch_info",
        )
        info = {"ntiles": nt.value, "order": ("given", "largest_first")[order.value], "wslots": ws.value,
                "raw_slots": raw.value, "tuned_ms": ms.value}
        n = ctypes.c_int()
        arrs = [(ctypes.c_int * 3)() for _ in range(6)]
        _check(lib().bf_batch_shape(self._h, ctypes.byref(n), *arrs), "bf_batch_shape")
        names = ("problems", "tiles", "max_nb_pass", "stages", "unpack_groups", "ctas_per_sm")
        info["launches"] = [{k: a[i] for k, a in zip(names, arrs)} for i in range(n.value)]
        return info

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().bf_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------- checksum


def tensor_peak_tflops(stream=None) -> float:
    """Measured dense E4M3 tcgen05 MMA rate of the current device (TFLOP/s)."""
    out = ctypes.c_double()
    _check(lib().bf_tensor_peak(ctypes.byref(out), _stream_handle(stream)), "bf_tensor_peak")
    return out.value


def dp4a_peak_per_s(stream=None) -> float:
    """Measured CUDA-core dp4a rate of the current device (lane operations/s)."""
    out = ctypes.c_double()
    _check(lib().bf_dp4a_peak(ctypes.byref(out), _stream_handle(stream)), "bf_dp4a_peak")
    return out.value


def adler32_host(data) -> int:
    """adler32 (adler32.c:7-20) of a host uint8 array, computed by the library."""
    a = np.ascontiguousarray(data, dtype=np.uint8)
    out = ctypes.c_uint32()
    _check(lib().bf_adler32_host(a.ctypes.data, a.nbytes, ctypes.byref(out)), "bf_adler32_host")
    return int(out.value)


def adler32_device(data, nbytes: int | None = None, stream=None) -> int:
    """adler32 (adler32.c:7-20) of a CUDA uint8 tensor, computed on the GPU."""
    n = data.numel() if nbytes is None else nbytes
    p, k = _ptr(data, np.uint8, n)
    if k != PTR_DEVICE:
        raise ValueError("adler32_device takes a CUDA tensor")
    out = ctypes.c_uint32()
    _check(lib().bf_adler32_device(p, n, ctypes.byref(out), _stream_handle(stream)), "bf_adler32_device")
    return int(out.value)


# ------------------------------------------------------- workload generator


def fill_random_device(dst, seed: int, stream_id: int, stream=None) -> None:
    p, k = _ptr(dst, np.uint8, 0, writable=True)
    if k != PTR_DEVICE:
        raise ValueError("fill_random_device takes a CUDA tensor")
    _check(lib().bf_fill_random_device(p, dst.numel(), seed, stream_id, _stream_handle(stream)), "fill_random_device")


def fill_random_host(dst: np.ndarray, seed: int, stream_id: int) -> None:
    p, _ = _ptr(dst, np.uint8, 0, writable=True)
    _check(lib().bf_fill_random_host(p, dst.nbytes, seed, stream_id), "fill_random_host")


def gains(dims: Dims) -> np.ndarray:
    """G from the reference setup()'s formula (arraysizes.cxx:31-32)."""
    G = np.empty(dims.gsize, dtype=np.float32)
    d = dims.c()
    _check(lib().bf_gains_host(ctypes.byref(d), G.ctypes.data), "bf_gains_host")
    return G


def seeded_host_inputs(dims: Dims, seed: int) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """Seeded workload in host memory: E (stream 0) and A (stream 1) uniform
    bytes, G from setup()'s formula."""
    E = np.empty(dims.esize, dtype=np.uint8)
    A = np.empty(dims.asize, dtype=np.uint8)
    fill_random_host(E, seed, 0)
    fill_random_host(A, seed, 1)
    return E, A, gains(dims)
