"""The drop-in boundary from C and C++: the header compiles as C11, and
tests/abi_caller.cpp -- a caller written like the reference's main
(cpu.cxx:48-67: sizes set once, std::vector storage, form_beams, then the
checksum of J) -- builds against include/beamform.h and libbeamform.so with
g++.  Without a GPU it must report BF_ERR_NO_DEVICE cleanly; on the GPU its
checksums must equal the oracle's."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
LIBDIR = os.path.join(ROOT, "beamforming_gb300")


def _have_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except ImportError:
        return False


@pytest.fixture(scope="module")
def caller(bflib, tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    exe = str(tmp_path_factory.mktemp("cpp") / "abi_caller")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", os.path.join(ROOT, "tests", "abi_caller.cpp"),
                    "-I", os.path.join(ROOT, "include"), "-L", LIBDIR, "-lbeamform", f"-Wl,-rpath,{LIBDIR}",
                    "-o", exe], check=True, capture_output=True, text=True)
    return exe


def test_header_compiles_as_c():
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-fsyntax-only", "-x", "c",
                    os.path.join(ROOT, "include", "beamform.h")], check=True, capture_output=True, text=True)


def test_cpp_caller_without_a_device(caller):
    if _have_gpu():
        pytest.skip("a GPU is present")
    r = subprocess.run([caller, "64", "2", "64", "2", "8", "1"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 2, r.stdout + r.stderr
    assert r.stdout.startswith("status 3 "), r.stdout


@pytest.mark.gpu
@pytest.mark.parametrize("shape,seed", [((256, 2, 128, 2, 40), 5), ((100, 3, 64, 2, 24), 7)])
def test_cpp_caller_matches_oracle(caller, oracle, shape, seed):
    od = oracle.Dims(*shape)
    E, A, G = oracle.seeded_inputs(od, seed)
    want = oracle.adler32(oracle.form_beams(od, E, A, G))
    r = subprocess.run([caller, *map(str, shape), str(seed)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = dict(line.split() for line in r.stdout.strip().splitlines())
    assert int(lines["adler32"], 16) == want
    assert int(lines["fused"], 16) == want
