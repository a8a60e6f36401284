"""The C++ host mirror (include/g5gpu.hpp) builds with g++ against the C ABI,
and, on a GPU, drives the reference's step loop bit-exactly against the oracle."""
import os
import subprocess

import pytest

from godunov_five_eq_gb300 import build as gbuild
from oracle import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = "/usr/local/cuda"


def build_driver(tmp_path):
    gbuild.build()
    oracle.build()
    exe = str(tmp_path / "shock_tube_driver")
    libdir = os.path.dirname(gbuild.LIB)
    odir = os.path.dirname(oracle.LIB_PATH)
    cmd = [
        "g++", "-O2", "-std=c++17", os.path.join(ROOT, "tests", "cpp", "shock_tube_driver.cpp"),
        f"-I{CUDA}/include", f"-L{libdir}", "-lg5gpu", f"-L{odir}", "-lg5oracle", f"-L{CUDA}/lib64", "-lcudart",
        f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{odir}", f"-Wl,-rpath,{CUDA}/lib64", "-o", exe,
    ]
    # the link name of the in-tree libraries
    for lib, d in ((gbuild.LIB, libdir), (oracle.LIB_PATH, odir)):
        name = os.path.basename(lib)
        assert name.startswith("lib") and name.endswith(".so")
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_cpp_host_mirror_builds(tmp_path):
    exe = build_driver(tmp_path)
    assert os.path.exists(exe)


@pytest.mark.gpu
def test_cpp_host_mirror_bit_exact_on_gpu(tmp_path):
    exe = build_driver(tmp_path)
    r = subprocess.run([exe, "12"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("OK")
