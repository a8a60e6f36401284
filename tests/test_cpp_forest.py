"""The C++ forest wrapper of include/g5gpu.hpp (g5::Forest) driven from a C++
program gives the same leaves, old -> new block map and block table as the
Python mesh (godunov_five_eq_gb300.mesh.BlockMesh) on the same refinement and
flags.  Host only: builds with g++ and runs without a GPU."""
import os
import subprocess

import numpy as np
import pytest

from godunov_five_eq_gb300 import build as gbuild
from godunov_five_eq_gb300.mesh import BlockMesh

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = "/usr/local/cuda"


def _driver(tmp_path):
    gbuild.build()
    exe = str(tmp_path / "forest_driver")
    libdir = os.path.dirname(gbuild.LIB)
    cmd = [
        "g++", "-O2", "-std=c++17", os.path.join(ROOT, "tests", "cpp", "forest_driver.cpp"),
        f"-I{CUDA}/include", f"-L{libdir}", "-lg5gpu", f"-L{CUDA}/lib64", "-lcudart",
        f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{CUDA}/lib64", "-o", exe,
    ]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def _parse(out):
    res = {}
    for line in out.strip().splitlines():
        name, *vals = line.split()
        res[name] = np.array([int(v) for v in vals[1:]] if name not in ("n_new", "sizes") else [int(v) for v in vals])
    return res


@pytest.mark.parametrize("dim,nbrick,periodic,lmin,lmax,seed", [(2, (3, 2, 1), False, 1, 4, 0), (3, (2, 1, 1), True, 0, 2, 1)])
def test_cpp_forest_matches_mesh(tmp_path, dim, nbrick, periodic, lmin, lmax, seed):
    exe = _driver(tmp_path)
    b = 8
    rng = np.random.default_rng(seed)
    mesh = BlockMesh(dim, b, nbrick[:dim], (periodic,) * dim, lmin, lmax)
    leaves = sorted(mesh.leaves)
    keys = [leaves[i] for i in rng.choice(len(leaves), size=min(3, len(leaves)), replace=False)]
    mesh.refine(keys)
    mesh.balance()
    order0 = mesh.ordered_leaves()
    flags = rng.choice(np.array([0, 1, 2], np.int8), size=len(order0), p=[0.5, 0.3, 0.2])
    rt = mesh.adapt(flags)
    t = mesh.build()
    spec = [dim, b, *[nbrick[e] if e < dim else 1 for e in range(3)], *[int(periodic) if e < dim else 0 for e in range(3)], lmin, lmax]
    text = " ".join(map(str, spec)) + f"\n{len(keys)}\n"
    text += "\n".join(" ".join(map(str, k)) for k in keys)
    text += f"\n{len(flags)}\n" + " ".join(map(str, flags.tolist())) + "\n"
    r = subprocess.run([exe], input=text, capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    got = _parse(r.stdout)
    assert np.array_equal(got["leaves0"].reshape(-1, 4), np.array(order0))
    assert got["n_new"][0] == rt.n_new
    assert np.array_equal(got["kind"], rt.kind) and np.array_equal(got["src"], rt.src.reshape(-1))
    assert tuple(got["sizes"]) == (t.n_owned, t.n_outside)
    for name in ("level", "coord", "nbr", "nbr_rel", "out_src", "out_normal", "out_border"):
        assert np.array_equal(got[name], getattr(t, name).reshape(-1)), name
