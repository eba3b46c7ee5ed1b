"""Build libcvortex.so in-tree (cvortex_gb300/lib/) for sm_103a.

CUDA translation units are compiled by nvcc with
``-gencode arch=compute_103a,code=sm_103a``; host C++ by the system g++ with
OpenMP. Objects are rebuilt only when a source or header is newer, and
translation units compile in parallel. No cmake, no torch extension machinery:
the product is a plain C-ABI shared library.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "lib"
OBJ = OUT / "obj"
LIB = OUT / "libcvortex.so"
INCLUDE = REPO / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), os.environ.get("CUDA_PATH"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _headers() -> list[Path]:
    hs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh"))
    hs += list((INCLUDE / "cvortex").glob("*.h")) + list((INCLUDE / "bsv").glob("*.h"))
    return hs


def _stale(src: Path, obj: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or newest_header > t


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def build(verbose: bool = False, ptxas_info: bool = False) -> Path:
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    OBJ.mkdir(parents=True, exist_ok=True)
    newest = max((h.stat().st_mtime for h in _headers()), default=0.0)
    inc = ["-I", str(INCLUDE), "-I", str(CSRC),
           '-DCVTX_EXPORT=__attribute__((visibility("default")))']
    cu_flags = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                "-Xcompiler", "-fPIC,-fopenmp,-fvisibility=hidden", *inc]
    if ptxas_info:
        cu_flags += ["-Xptxas", "-v"]
    cxx = os.environ.get("CXX", "g++")
    cpp_flags = [cxx, "-O3", "-fPIC", "-fopenmp", "-fvisibility=hidden", "-std=c++17", "-Wall",
                 "-ffp-contract=off",
                 "-Wno-unused-function",
                 *inc, "-I", str(cuda / "include")]
    jobs = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp")):
        obj = OBJ / (src.name + ".o")
        objs.append(obj)
        if ptxas_info or _stale(src, obj, newest):
            base = cu_flags if src.suffix == ".cu" else cpp_flags
            jobs.append(base + ["-c", str(src), "-o", str(obj)])
    if jobs:
        workers = min(len(jobs), max(1, os.cpu_count() or 1))
        with cf.ThreadPoolExecutor(workers) as ex:
            futs = [ex.submit(_run_capture if ptxas_info else _run, j) for j in jobs]
            for f in futs:
                out = f.result()
                if ptxas_info and out:
                    sys.stdout.write(out)
    if jobs or not LIB.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs),
              "-Xcompiler", "-fopenmp", "-lgomp"])
    if verbose:
        print(f"built {LIB}")
    return LIB


def _run_capture(cmd: list[str]) -> str:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)
    return res.stdout + res.stderr


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
