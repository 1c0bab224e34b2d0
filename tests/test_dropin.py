"""The C++ drop-in (include/CANDMC.h): a reference-style program written against
the reference's signatures compiles and links against the library (CPU), and
passes the reference tests' criteria on the GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "dropin", "test_dropin.cxx")
LIBDIR = os.path.join(ROOT, "candmc_gb300")


def _compile(tmp_path):
    from candmc_gb300 import build
    build.build()
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "test_dropin")
    cmd = [cxx, "-O2", "-std=c++17", SRC, "-I", os.path.join(ROOT, "include"),
           "-I", "/usr/local/cuda/include", "-L", LIBDIR, "-lcandmc_gb300",
           f"-Wl,-rpath,{LIBDIR}", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_dropin_program_compiles_and_links(tmp_path):
    assert os.path.exists(_compile(tmp_path))


@pytest.mark.gpu
def test_dropin_program_passes_reference_criteria(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    exe = _compile(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "TEST FAILED" not in r.stdout
    assert r.stdout.count("Test successful.") == 12
