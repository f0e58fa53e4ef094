"""GPU: the sample programs (tests/samples/*.cpp), written against the C++ host
surface include/hipacc_gb300/hipacc.hpp in the shape of the reference's
samples, compile with g++, link libhipacc_gb300.so and pass their own checks."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SAMPLES = ["gaussian_blur", "sobel", "color_reduce", "pyramid", "bilateral", "graph", "pipelines"]


@pytest.fixture(scope="module")
def binaries(hgb_lib):
    out = os.path.join(ROOT, "tests", "samples", "bin")
    os.makedirs(out, exist_ok=True)
    libdir = os.path.join(ROOT, "hipacc_gb300")
    built = {}
    for name in SAMPLES:
        exe = os.path.join(out, name)
        cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"),
               os.path.join(ROOT, "tests", "samples", name + ".cpp"), "-L", libdir, "-lhipacc_gb300",
               "-Wl,-rpath," + libdir, "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        built[name] = exe
    return built


@pytest.mark.parametrize("name", SAMPLES)
def test_sample(binaries, gpu, name):
    r = subprocess.run([binaries[name]], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Test PASSED" in r.stdout
