"""Build libmtr (CUDA kernels + C ABI + MRC/TXBR/options I/O) and the
mtr_multiaxis command-line tool, in-tree, for sm_103a only.

Plain nvcc / g++ invocations run in parallel; a target is rebuilt only when
one of its sources or headers is newer.  Outputs:
    lib/libmtr.so          the C-ABI shared library (static CUDA runtime)
    bin/mtr_multiaxis      the drop-in command-line program
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
OBJ = PKG / "_build"
LIB = PKG / "lib"
BIN = PKG / "bin"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=default",
                     "--expt-relaxed-constexpr", "-I", str(INCLUDE)]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function", "-I", str(INCLUDE)]

CU_SOURCES = ["projector.cu", "bp_tma.cu", "fwd_tma.cu", "mace.cu", "api.cu", "recon.cu", "entry.cu", "ref64.cu",
              "noalloc.cu", "tune.cu", "batch.cu", "serve.cu", "mrc_device.cu", "stream.cu", "bp_pairs.cu"]
CXX_SOURCES = ["mrc_io.cpp", "options.cpp", "geometry.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libmtr")


def _headers() -> list[Path]:
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, jobs: int | None = None) -> dict:
    OBJ.mkdir(exist_ok=True)
    LIB.mkdir(exist_ok=True)
    BIN.mkdir(exist_ok=True)
    hdrs = _headers()
    steps = []
    objs = []
    for s in CU_SOURCES:
        src, obj = CSRC / s, OBJ / (s + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            steps.append([nvcc()] + NVCC_FLAGS + ["-c", str(src), "-o", str(obj)])
    for s in CXX_SOURCES + ["cli_main.cpp"]:
        src, obj = CSRC / s, OBJ / (s + ".o")
        if s != "cli_main.cpp":
            objs.append(obj)
        if _stale(obj, [src] + hdrs):
            steps.append(["g++"] + CXX_FLAGS + ["-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        for f in [ex.submit(_run, c) for c in steps]:
            f.result()
    lib = LIB / "libmtr.so"
    if _stale(lib, objs):
        _run([nvcc()] + ARCH + ["-shared", "-o", str(lib)] + [str(o) for o in objs])
    cli = BIN / "mtr_multiaxis"
    cli_obj = OBJ / "cli_main.cpp.o"
    if _stale(cli, [cli_obj, lib]):
        _run(["g++", "-o", str(cli), str(cli_obj), "-L", str(LIB), "-lmtr", "-Wl,-rpath,$ORIGIN/../lib"])
    if verbose:
        print(f"libmtr: {len(steps)} compile step(s); {lib}")
    return {"lib": str(lib), "cli": str(cli)}


if __name__ == "__main__":
    print(build(verbose=True))
