"""The C++ facades (include/spectrum_gb300/spectrum.hpp) through a C++ test
program written against the reference's class names: it is compiled with the
system C++ compiler against the in-tree library and run; every check prints
PASS/FAIL and the program exits non-zero on any failure."""
import os
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "facade_kat.cpp"
LIB = ROOT / "spectrum_gb300" / "lib"
CUDA = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def _compile(out: Path) -> Path:
    if not (LIB / "libspectrum_gb300.so").exists():
        pytest.fail("native library not built")
    cxx = os.environ.get("CXX", "g++")
    cmd = [cxx, "-std=c++17", "-O1", "-Wall", str(SRC), f"-I{ROOT / 'include'}", f"-I{CUDA / 'include'}",
           f"-L{LIB}", "-lspectrum_gb300", f"-L{CUDA / 'lib64'}", "-lcudart",
           f"-Wl,-rpath,{LIB}:{CUDA / 'lib64'}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def _run(exe: Path, *args) -> str:
    r = subprocess.run([str(exe), *args], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    last = r.stdout.strip().splitlines()[-1].split()
    assert last[0] == "SUMMARY" and int(last[2]) == 0 and int(last[1]) > 0
    return r.stdout


def test_facades_compile_against_reference_names_and_refuse_without_gpu(tmp_path):
    """Compiles here (no GPU) and checks that construction without a device
    raises std::runtime_error and a null backend std::invalid_argument."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("covered by the GPU run of the same program")
    _run(_compile(tmp_path / "facade_kat"), "--no-gpu")


@pytest.mark.gpu
def test_facade_known_answers_on_gpu(tmp_path, spx):
    out = _run(_compile(tmp_path / "facade_kat"))
    assert "FAIL" not in out
    assert out.count("PASS") >= 30
