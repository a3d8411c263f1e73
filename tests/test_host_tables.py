"""Host-side tables of libqsg.so checked on the CPU (tests/cpp/host_tables.cpp):
the Bluestein chirp and FFT_M(conj chirp) / M of the long buffers, formed in
double-double arithmetic (blue_tables_dd), against the long double tables of
the one-CTA kernels and against a direct DFT at small sizes."""
import json
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "host_tables.cpp")
EXE = os.path.join(ROOT, "tests", "cpp", "host_tables")

pytestmark = pytest.mark.skipif(shutil.which("g++") is None, reason="no C++ compiler")


@pytest.fixture(scope="module")
def tables():
    from qusim_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    cuda = "/usr/local/cuda"
    subprocess.run(["g++", "-std=c++17", "-O2", SRC, "-o", EXE, "-L", libdir, "-lqsg", f"-Wl,-rpath,{libdir}",
                    "-L", os.path.join(cuda, "lib64"), f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}", "-lcudart"],
                   check=True)
    out = subprocess.run([EXE], capture_output=True, text=True, check=True, timeout=300).stdout
    return json.loads(out.strip().splitlines()[-1])


def test_double_double_tables_match_long_double(tables):
    for key, (dw, dh, ddft) in tables.items():
        # both round to double at the end: half an ulp apart at most, relative to the largest entry
        assert dw <= 3e-16, key
        assert dh <= 3e-16, key


def test_double_double_tables_match_a_direct_dft(tables):
    for key in ("3_8", "100_256", "1000_2048"):
        assert tables[key][2] <= 3e-16, key
