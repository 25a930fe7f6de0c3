"""Build recipe for the native library (nvcc, sm_103a only).

Compiles every ``csrc/*.cu`` translation unit in parallel into
``spectrum_gb300/_build/`` and links ``spectrum_gb300/lib/libspectrum_gb300.so``.
Used by ``__graft_entry__.build()`` and by ``python -m spectrum_gb300._build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libspectrum_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build spectrum_gb300")
    return cand


def _flags(ptxas_verbose: bool) -> list[str]:
    f = ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
        "-Xcompiler", "-fPIC,-O2",
        f"-I{ROOT / 'include'}", f"-I{CSRC}",
    ]
    if ptxas_verbose:
        f += ["-Xptxas", "-v"]
    return f


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _compile_one(src: Path, ptxas_verbose: bool) -> tuple[Path, str]:
    obj = BUILD / (src.stem + ".o")
    deps = [src] + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted((ROOT / "include").rglob("*.h*"))
    if obj.exists() and not ptxas_verbose:
        t = obj.stat().st_mtime
        if all(d.stat().st_mtime <= t for d in deps if d.exists()):
            return obj, ""
    cmd = [nvcc(), "-c", str(src), "-o", str(obj)] + _flags(ptxas_verbose)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stdout + r.stderr


def build(verbose: bool = False, ptxas_verbose: bool = False) -> Path:
    """Compiles and links the library; returns the path of the .so."""
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(lambda s: _compile_one(s, ptxas_verbose), srcs))
    objs = [o for o, _ in results]
    if verbose or ptxas_verbose:
        for o, log in results:
            if log:
                print(f"--- {o.name}\n{log}", file=sys.stderr)
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), "-shared", "-o", str(tmp)] + [str(o) for o in objs] + ARCH + [
            "-cudart", "shared", "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    p = build(verbose=True, ptxas_verbose="-v" in sys.argv)
    print(p)
