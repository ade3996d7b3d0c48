"""Build recipe for libbms.so (sm_103a kernels + C ABI) and the CPU oracle.

Everything is compiled in-tree into ``bms2_gb300/_build/`` and ``oracle/_build/``
with plain nvcc / g++ invocations run in parallel (no cmake).  Host code avoids
architecture-specific flags so the same sources build on x86_64 and aarch64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libbms.so"
CLI = OUT / "bms2"
ORACLE_DIR = ROOT / "oracle"
ORACLE_OUT = ORACLE_DIR / "_build"
ORACLE_LIB = ORACLE_OUT / "liboracle.so"
# the workload generator alone, for the CPU side (no engine code mapped there)
SYNTH_LIB = ORACLE_OUT / "libsynth.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _nvcc() -> str:
    cand = Path(CUDA_HOME) / "bin" / "nvcc"
    return str(cand) if cand.exists() else (shutil.which("nvcc") or "nvcc")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + res.stdout + res.stderr)


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, jobs: int | None = None) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "bms.h"]
    units = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    nvcc = _nvcc()
    inc = ["-I", str(ROOT / "include"), "-I", str(CSRC)]
    jobs_ = []
    objs = []
    for src in units:
        obj = OUT / (src.name + ".o")
        objs.append(obj)
        if not force and not _stale(obj, [src] + headers):
            continue
        if src.suffix == ".cu":
            cmd = [nvcc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
                   *inc, "-c", str(src), "-o", str(obj)]
        else:
            cmd = [nvcc, "-std=c++17", "-O2", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", *inc, "-c", str(src),
                   "-o", str(obj)]
        jobs_.append(cmd)
    if jobs_:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(jobs_), os.cpu_count() or 4)) as ex:
            list(ex.map(_run, jobs_))
    if force or jobs_ or _stale(LIB, objs):
        _run([nvcc, "-shared", *ARCH, "-cudart", "static", "-o", str(LIB), *map(str, objs), "-lpthread", "-ldl",
              "-lrt"])
    cli_src = CSRC / "tools" / "bms2_main.cpp"
    if force or _stale(CLI, [cli_src, LIB, ROOT / "include" / "bms.hpp", ROOT / "include" / "bms.h"]):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(cli_src), "-o", str(CLI), "-L", str(OUT),
              "-lbms", "-Wl,-rpath,$ORIGIN"])
    return LIB


def build_oracle(force: bool = False) -> Path:
    ORACLE_OUT.mkdir(parents=True, exist_ok=True)
    src = ORACLE_DIR / "oracle.cpp"
    if force or _stale(ORACLE_LIB, [src]):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-std=c++17", "-O3", "-fopenmp", "-fPIC", "-shared", str(src), "-o", str(ORACLE_LIB)])
    return ORACLE_LIB


def build_synth(force: bool = False) -> Path:
    """The seeded generator (csrc/synth.cpp with its host graph container
    csrc/graphs.cpp) compiled on its own, without CUDA, for the CPU baseline."""
    ORACLE_OUT.mkdir(parents=True, exist_ok=True)
    srcs = [CSRC / "synth.cpp", CSRC / "graphs.cpp"]
    deps = srcs + [CSRC / "graphs.h", ROOT / "include" / "bms.h"]
    if force or _stale(SYNTH_LIB, deps):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-std=c++17", "-O2", "-fPIC", "-shared", "-I", str(ROOT / "include"), *map(str, srcs), "-o",
              str(SYNTH_LIB), "-lpthread"])
    return SYNTH_LIB


def build_cpu_side(force: bool = False) -> None:
    """What the CPU-baseline arm needs: the oracle and the generator."""
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        for f in [ex.submit(build_oracle, force), ex.submit(build_synth, force)]:
            f.result()


def build(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        fs = [ex.submit(build_library, force), ex.submit(build_oracle, force), ex.submit(build_synth, force)]
        for f in fs:
            f.result()


if __name__ == "__main__":
    import sys

    build(force="--force" in sys.argv)
    print(LIB)
