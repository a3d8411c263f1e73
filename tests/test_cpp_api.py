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
    # the same run from the reference's expression strings (FunctorWrapper), and a Calculator
    assert abs(r["transmission_expr"] - r["transmission"]) < 1e-12
    assert abs(complex(*r["calculator"]) - (18 + 1j)) < 1e-13  # x^2 through complex pow, as in the reference


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 2e-5)])
def test_cpp_api_born_series_against_oracle(exe, oracle, precision, tol):
    """QuPerturbation1D / 2D through the C++ API equal the oracle's series."""
    import numpy as np
    out = subprocess.run([exe, precision], capture_output=True, text=True, check=True).stdout
    r = json.loads(out.strip().splitlines()[-1])
    x = -100 + 200 / 2048 * np.arange(2048)
    ref = oracle.born1d(0.5 * np.exp(-x * x) + 0j, -100.0, 100.0, 0.5, 0.51, order=5, preconditional=True)
    assert abs(r["born_R"] - ref["R"]) <= tol and abs(r["born_T"] - ref["T"]) <= tol
    assert r["born_eps"] == ref["epsilon"]
    g = -45 + 90 / 128 * np.arange(128)
    X, Y = np.meshgrid(g, g, indexing="ij")
    ref2 = oracle.born2d(0.3 * np.exp(-(X * X + Y * Y) / 4) + 0j, -45.0, 45.0, -45.0, 45.0, 2.0, 0.0, dirx=1.0,
                         diry=0.0, order=3, preconditional=True, preconditioner=3, slow=0.5, cosxy=[(1.0, 0.0)])
    assert abs(r["born2d_xsec0"] - ref2["xsec"][0]) <= 10 * tol * ref2["xsec"][0]
    assert abs(r["born2d_delta"] - ref2["delta_norm"]) <= 10 * tol * ref2["delta_norm"]
