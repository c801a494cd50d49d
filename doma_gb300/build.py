"""Build the native library in-tree: doma_gb300/_lib/libdoma_gb300.so.

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, then linked with the
host objects into one shared library against the shared CUDA runtime.  Host
code is compiled with -ffp-contract=off: the FP64 drop-in mode relies on
unfused, separately rounded host arithmetic (the quadrature) as well.

Usage: python -m doma_gb300.build [--verbose-ptxas]
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
SRC = PKG / "csrc"
OUT = PKG / "_lib"
OBJ = OUT / "obj"
LIB = OUT / "libdoma_gb300.so"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["sweep.cu", "iteration.cu", "solver.cu", "noalloc.cu", "conv.cu", "conv_tc.cu", "unet.cu", "accel.cu"]
CPP_SOURCES = ["quadrature.cpp"]

# C++ drop-in layer (DOMA's TransportSolver3D/2D, BrickMesh3D/2D and
# InputParameters interface) over the C ABI, and the deck runner.
HOST = PKG / "host"
HOST_SOURCES = ["xml.cpp", "InputParameters.cpp", "BrickMesh.cpp", "TransportSolver.cpp"]
HOST_LIB = OUT / "libdoma_gb300_host.so"
CLI = OUT / "doma_gb300"


def _nvcc() -> str:
    p = CUDA_HOME / "bin" / "nvcc"
    return str(p) if p.exists() else (shutil.which("nvcc") or "nvcc")


def _run(cmd: list[str]) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed ({r.returncode}): {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(verbose_ptxas: bool = False, force: bool = False) -> Path:
    OBJ.mkdir(parents=True, exist_ok=True)
    headers = sorted(SRC.glob("*.cuh")) + [PKG.parent / "include" / "doma_gb300.h"]
    nvcc = _nvcc()
    jobs = []
    for name in CU_SOURCES:
        src = SRC / name
        obj = OBJ / (name + ".o")
        if force or verbose_ptxas or _stale(obj, [src, *headers]):
            cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-c", str(src), "-o", str(obj),
                   "-Xcompiler", "-fPIC,-ffp-contract=off", "--expt-relaxed-constexpr"]
            if verbose_ptxas:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    for name in CPP_SOURCES:
        src = SRC / name
        obj = OBJ / (name + ".o")
        if force or _stale(obj, [src, *headers]):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off",
                         f"-I{CUDA_HOME / 'include'}", "-c", str(src), "-o", str(obj)])
    logs = []
    if jobs:
        with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            logs = list(ex.map(_run, jobs))
    objs = [str(OBJ / (n + ".o")) for n in CU_SOURCES + CPP_SOURCES]
    relinked = False
    if force or jobs or not LIB.exists():
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *objs, "-cudart", "shared",
              "-Xlinker", f"-rpath,{CUDA_HOME / 'lib64'}"])
        relinked = True
    build_host(force=force or relinked)
    if verbose_ptxas:
        for log in logs:
            sys.stdout.write(log)
    return LIB


def build_host(force: bool = False) -> Path:
    """libdoma_gb300_host.so (C++ drop-in classes) and the doma_gb300 CLI."""
    inc = [f"-I{HOST / 'include'}", f"-I{PKG.parent / 'include'}"]
    srcs = [HOST / "src" / n for n in HOST_SOURCES]
    deps = srcs + sorted((HOST / "include" / "doma").glob("*.h")) + sorted((HOST / "src").glob("*.h"))
    deps.append(PKG.parent / "include" / "doma_gb300.h")
    rpath = f"-Wl,-rpath,$ORIGIN,-rpath,{CUDA_HOME / 'lib64'}"
    if force or _stale(HOST_LIB, deps):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", *inc, *map(str, srcs), "-o", str(HOST_LIB),
              f"-L{OUT}", "-ldoma_gb300", rpath])
    main_src = HOST / "src" / "doma_main.cpp"
    if force or _stale(CLI, [main_src, HOST_LIB]):
        _run(["g++", "-O2", "-std=c++17", *inc, str(main_src), "-o", str(CLI), f"-L{OUT}",
              "-ldoma_gb300_host", "-ldoma_gb300", rpath])
    return HOST_LIB


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--verbose-ptxas", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build(verbose_ptxas=a.verbose_ptxas, force=a.force))


if __name__ == "__main__":
    main()
