"""The C++ host API (include/qusim_gb300/Evolver.h): it compiles and links
against libqsg.so here (CPU); on a GPU it reproduces the reference's
tunnelling known answer (QuSimPrecision.cpp:82)."""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "evolver_api.cpp")
EXE = os.path.join(ROOT, "tests", "cpp", "evolver_api")


@pytest.fixture(scope="module")
def exe():
    from qusim_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    cuda = "/usr/local/cuda"
    cmd = ["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), SRC, "-o", EXE,
           "-L", libdir, "-lqsg", f"-Wl,-rpath,{libdir}", "-L", os.path.join(cuda, "lib64"),
           f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}", "-lcudart"]
    subprocess.run(cmd, check=True)
    return EXE


def test_cpp_api_builds(exe):
    assert os.access(exe, os.X_OK)


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("mixed", 2e-6)])
def test_cpp_api_tunnelling_known_answer(exe, precision, tol):
    out = subprocess.run([exe, precision], capture_output=True, text=True, check=True).stdout
    r = json.loads(out.strip().splitlines()[-1])
    ref = (0.1593774409 + 0.1593774408) / 2
    # complex64 state: the initial norm carries the float rounding of psi0
    assert abs(r["norm0"] - 1) < (1e-12 if precision == "fp64" else 1e-7)
    assert abs(r["time"] - 64.0) < 1e-9
    assert abs(r["transmission"] - ref) < tol
    assert abs(r["norm2d"] - 1) < 1e-5
    assert r["wall2d_throws"] and r["bad_device_throws"]
