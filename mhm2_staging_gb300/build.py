"""Build recipe for the native libraries of this package (in-tree, no CMake).

Outputs (git-ignored, under mhm2_staging_gb300/_build/):
  libmhsw.so      the CUDA kernels + host driver behind include/mhsw.h (sm_103a)
  libmhsw_gen.so  seeded synthetic workload generators (host C++)
  klign_block_bench  klign's GPU call sequence through the C++ drop-in header
                  (include/adept-sw/driver.hpp) on 20,000-pair blocks, timed (bench.py)

Translation units are compiled in parallel; a unit is rebuilt only when its source or
any header in csrc/ or include/ is newer than its object.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_UNITS = ["mhsw_kernels.cu", "mhsw_batch.cu", "mhsw_driver.cu", "mhsw_probe.cu", "mhsw_noalloc.cu", "mhsw_cigar.cu", "mhsw_klign.cu", "mhsw_protein.cu",
              "mhsw_server.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmhsw.so")


def _headers_mtime() -> float:
    files = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return max((f.stat().st_mtime for f in files), default=0.0)


def _stale(out: Path, srcs: list[Path], hdr_mtime: float) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(s.stat().st_mtime > t for s in srcs) or hdr_mtime > t


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, jobs: int | None = None) -> dict[str, Path]:
    BUILD.mkdir(parents=True, exist_ok=True)
    nvcc = _nvcc()
    hdr = _headers_mtime()
    cflags = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I", str(INCLUDE)]
    jobs = jobs or min(8, os.cpu_count() or 4)

    def compile_cu(name: str) -> Path:
        src = CSRC / name
        obj = BUILD / (Path(name).stem + ".o")
        if _stale(obj, [src], hdr):
            cmd = [nvcc, *ARCH_FLAGS, *cflags, "-c", str(src), "-o", str(obj)]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            _run(cmd)
        return obj

    def build_gen() -> Path:
        src = CSRC / "gen_workloads.cpp"
        out = BUILD / "libmhsw_gen.so"
        if _stale(out, [src], 0.0):
            cxx = os.environ.get("CXX", "g++")
            _run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-pthread", "-o", str(out), str(src)])
        return out

    with ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(compile_cu, u) for u in CUDA_UNITS]
        gen_f = ex.submit(build_gen)
        objs = [f.result() for f in futs]
        gen = gen_f.result()

    lib = BUILD / "libmhsw.so"
    if _stale(lib, objs, 0.0):
        _run([nvcc, *ARCH_FLAGS, "-shared", "-o", str(lib), *map(str, objs), "-cudart", "static"])
    bench = BUILD / "klign_block_bench"
    bsrc = CSRC / "klign_block_bench.cpp"
    if _stale(bench, [bsrc, lib], hdr):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-O2", "-std=c++14", "-I", str(INCLUDE), str(bsrc), "-o", str(bench), str(lib),
              f"-Wl,-rpath,{BUILD}"])
    return {"libmhsw": lib, "libmhsw_gen": gen, "klign_block_bench": bench}


def lib_path() -> Path:
    return BUILD / "libmhsw.so"


def gen_lib_path() -> Path:
    return BUILD / "libmhsw_gen.so"


def block_bench_path() -> Path:
    return BUILD / "klign_block_bench"


if __name__ == "__main__":
    out = build(verbose="-v" in sys.argv)
    for k, v in out.items():
        print(k, v)
