"""Build libwatercube.so in-tree for sm_103a (nvcc, one -gencode, objects compiled in parallel).

The solver is the CUDA sources under csrc/ plus the host-only C++ in csrc/*.cpp, linked into
watercube_gb300/libwatercube.so next to this file (git-ignored). No CMake, no torch.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
REPO = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libwatercube.so"

NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    *ARCH,
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "-Xcompiler",
    "-fPIC,-fvisibility=hidden,-ffp-contract=off",
    "--expt-relaxed-constexpr",
    f"-I{REPO / 'include'}",
]
CXX_FLAGS = ["-O2", "-fPIC", "-fvisibility=hidden", "-ffp-contract=off", "-std=c++17", f"-I{REPO / 'include'}"]


def _cuda_include() -> str:
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    return str(Path(home) / "include")


def _sources():
    return sorted(CSRC.glob("*.cu")), sorted(CSRC.glob("*.cpp"))


def _stale(lib: Path) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = list(CSRC.glob("*")) + [REPO / "include" / "watercube.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.is_file())


def build(force: bool = False, verbose: bool = False, ptxas_info: bool = False) -> Path:
    if not force and not _stale(LIB):
        return LIB
    BUILD.mkdir(exist_ok=True)
    cus, cpps = _sources()
    jobs = []
    for src in cus:
        extra = ["-Xptxas", "-v"] if ptxas_info else []
        jobs.append([NVCC, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(BUILD / (src.stem + ".o"))])
    for src in cpps:
        jobs.append(["g++", *CXX_FLAGS, f"-I{_cuda_include()}", "-c", str(src), "-o", str(BUILD / (src.stem + ".o"))])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode:
            raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stdout + r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        logs = list(ex.map(run, jobs))
    if verbose or ptxas_info:
        for log in logs:
            if log.strip():
                print(log, file=sys.stderr)
    objs = [str(BUILD / (s.stem + ".o")) for s in cus + cpps]
    tmp = LIB.with_suffix(".so.tmp")
    run([NVCC, *ARCH, "-shared", "-o", str(tmp), *objs, "-cudart", "static"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, verbose=True, ptxas_info=a.ptxas_info))
