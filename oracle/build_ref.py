"""Builds the reference-derived checkers into oracle/_ref/ (TEST INFRASTRUCTURE ONLY).

Only where the reference sources are present (this development container;
the GPU machine has none and never needs them).  Two shared libraries, both
compiled from the reference's sources where they lie, nothing copied into
the repository:

* ``oracle/_ref/libref_cpufft.so`` — the reference's ``spectrum_utils::CpuFFT``
  (include/spectrum/utils/cpu_fft.hpp + its vendored third_party/pocketfft),
  through ``oracle/ref_cpufft_shim.cpp``;
* ``oracle/_ref/libref_kernels.so`` — the reference's own peak-search and
  magnitude kernel text, extracted from its kernel-source headers by
  ``oracle/ref_kernel_dump.cpp`` and executed on the CPU by the fiber
  harness ``oracle/ref_simt.h`` / ``oracle/ref_kernels_host.cpp``.

Plain g++ on those few files, no build system of the reference.  FP
contraction is disabled so ``x*x + y*y`` rounds each operation, as numpy does.
The reference's location comes from the caller (``build(root)``,
``reference_present(root)``) or from the SPX_REFERENCE_ROOT environment
variable; this file assumes no path of its own.
"""
from __future__ import annotations

import os
import re
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"

CXX = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math"]


def _root(root) -> Path | None:
    r = root or os.environ.get("SPX_REFERENCE_ROOT")
    return Path(r) if r else None


def reference_present(root=None) -> bool:
    ref = _root(root)
    return ref is not None and (ref / "include" / "spectrum" / "utils" / "cpu_fft.hpp").exists() and \
        (ref / "include" / "spectrum" / "kernels" / "all_maxima_kernel_sources_rocm.hpp").exists()


def _run(cmd):
    r = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")
    return r


def _sanitize(text: str) -> str:
    """Makes kernel text compile as host C++ under ref_simt.h: drop the C
    linkage (each source is wrapped in its own namespace) and point the one
    dynamic shared-memory array at the harness's buffer."""
    text = text.replace('extern "C"', "")
    text = re.sub(r"extern\s+__shared__\s+unsigned\s+int\s+(\w+)\s*\[\s*\]\s*;",
                  r"unsigned int* \1 = static_cast<unsigned int*>(ref_simt_dynamic_smem());", text)
    return text


def build(root=None, force: bool = False) -> dict:
    ref = _root(root)
    if not reference_present(ref):
        raise FileNotFoundError(f"reference sources not found under {ref} (give root or SPX_REFERENCE_ROOT)")
    OUT.mkdir(exist_ok=True)
    inc = ref / "include"
    pocket = ref / "third_party" / "pocketfft"
    libs = {"cpufft": OUT / "libref_cpufft.so", "kernels": OUT / "libref_kernels.so"}

    def stale(lib: Path, *srcs: Path) -> bool:
        return force or not lib.exists() or any(src.stat().st_mtime > lib.stat().st_mtime for src in srcs)

    if stale(libs["cpufft"], HERE / "ref_cpufft_shim.cpp"):
        _run(CXX + ["-shared", "-fPIC", f"-I{inc}", f"-I{pocket}", HERE / "ref_cpufft_shim.cpp",
                    "-o", libs["cpufft"]])

    if stale(libs["kernels"], HERE / "ref_kernels_host.cpp", HERE / "ref_simt.h", HERE / "ref_kernel_dump.cpp"):
        dump = OUT / "ref_kernel_dump"
        _run(CXX + ["-DENABLE_ROCM=1", f"-I{inc}", HERE / "ref_kernel_dump.cpp", "-o", dump])
        raw = [OUT / "spectrum.txt", OUT / "allmax.txt", OUT / "fftproc.txt"]
        _run([dump] + raw)
        for src, name in zip(raw, ["gen_spectrum.inc", "gen_allmax.inc", "gen_fftproc.inc"]):
            (OUT / name).write_text(_sanitize(src.read_text()))
        _run(CXX + ["-shared", "-fPIC", f"-I{HERE}", f"-I{OUT}", HERE / "ref_kernels_host.cpp",
                    "-o", libs["kernels"]])
    return libs


if __name__ == "__main__":
    import sys
    print(build(sys.argv[1] if len(sys.argv) > 1 else None, force=True))
