"""The reference-side binding (tests/cpp/ref_binding.cpp) compiled against the
reference's own unmodified headers (src/EvolverImpl.h, OptionsImpl.h,
DeviceType.h, SplittingMethod1D/2D.h) and linked with its own objects
(oracle/_ref) and libqsg.so.

It exercises the implementation choice of Evolver1D/2D::init
(src/QuSim.cpp:90-100, 161-169) with the GPU_GB300 branch added:
  - "CPU_SEQ" selects the reference's SplittingMethod1D/2D, which reproduce
    the tunnelling known answer 0.15937744085
    (applications/QuEvol1DPrecision/QuSimPrecision.cpp:82);
  - "GPU_GB300" selects the engine's QuEvolverImpl subclasses: on a machine
    with a GPU they give the same numbers to 1e-12 (complex128); without one
    the engine's failure surfaces as the std::runtime_error the reference
    raises for device errors;
  - an unknown device still reaches GetDeviceType (src/DeviceType.h:9-22) and
    raises std::invalid_argument.
Needs the reference source tree (QUSIM_REF, default /root/reference); the
test is skipped where it is absent.
"""
import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.environ.get("QUSIM_REF", "/root/reference")
SRC = os.path.join(ROOT, "tests", "cpp", "ref_binding.cpp")
EXE = os.path.join(ROOT, "tests", "cpp", "ref_binding")
REF_OBJS = ["EvolverImpl", "EvolverImpl1D", "EvolverImpl2D", "SplittingMethod1D", "SplittingMethod2D",
            "SplittingUtils", "FourierTransform", "Device", "OptionsImpl", "fftw_stub"]
KNOWN = (0.1593774409 + 0.1593774408) / 2

pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF, "src")),
                                reason="reference source tree not present")


@pytest.fixture(scope="module")
def exe():
    from qusim_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "-j8", "ref", f"REF={REF}"], check=True)
    cuda = "/usr/local/cuda"
    objs = [os.path.join(ROOT, "oracle", "_ref", o + ".o") for o in REF_OBJS]
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-include", "cstdint", "-include", "stdexcept",
           "-include", "cstring", "-include", "string", "-include", "memory", "-DQUEXPORT", "-DEXPORT_FUNC=",
           "-DEXPORT_STRUCT=", "-I", os.path.join(REF, "include"), "-I", os.path.join(REF, "src"),
           "-I", os.path.join(ROOT, "oracle", "ref_shim"), "-I", os.path.join(ROOT, "include"), "-w", SRC, *objs,
           "-o", EXE, "-L", libdir, "-lqsg", f"-Wl,-rpath,{libdir}", "-L", os.path.join(cuda, "lib64"),
           f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}", "-lcudart"]
    subprocess.run(cmd, check=True)
    return EXE


def run(exe, *args):
    out = subprocess.run([exe, *args], capture_output=True, text=True, check=True, timeout=600).stdout
    return json.loads(out.strip().splitlines()[-1])


def gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_reference_device_through_the_new_factory(exe):
    r = run(exe, "CPU_SEQ")
    assert abs(r["time"] - 64.0) < 1e-9
    assert abs(r["norm0"] - 1) < 1e-12
    assert abs(r["transmission"] - KNOWN) < 1e-9
    assert abs(r["norm2d"] - 1) < 1e-12


def test_unknown_device_still_refused_by_get_device_type(exe):
    r = run(exe, "NO_SUCH_DEVICE")
    assert "invalid device" in r["invalid_argument"]


def test_gb300_device_selected(exe):
    r = run(exe, "GPU_GB300")
    if not gpu_present():
        # the engine was selected and its failure became the reference's exception
        assert r["runtime_error"].startswith("GPU_GB300:")
        return
    ref = run(exe, "CPU_SEQ")
    for k in ("norm0", "time", "transmission", "kin", "pot", "psi_1000_re", "norm2d", "kin2d", "pot2d", "psi2d_re",
              "psi2d_im"):
        assert abs(r[k] - ref[k]) <= 1e-12 * max(1.0, abs(ref[k])), k
