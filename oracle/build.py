"""Build recipe for the oracle, which is test infrastructure (never part of the product):

  oracle/liboracle.so        CPU restatement of the reference's math (oracle.cpp)
  oracle/liborc_refrun.so    harness that runs the reference's own kernels
                             from oracle/_ref/ref_kernels.cubin (ref_runner.cu)
and, only where the reference sources are present (elsewhere the prebuilt,
git-ignored oracle/_ref/ files are used):
  oracle/_ref/ref_kernels.cubin   the reference's FunctionOnGPU.cu, unmodified,
                                  device code for sm_103a
  oracle/_ref/ref_golden          golden-vector generator linked from the
                                  reference's CPU I/O sources (ref_golden.cpp)

The reference's own build system is not used: each piece is one nvcc/g++
command on the reference's files where they lie.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import subprocess
from pathlib import Path

ORACLE = Path(__file__).resolve().parent
REF_OUT = ORACLE / "_ref"
REFERENCE = Path(os.environ.get("MTR_REFERENCE_DIR", "/root/reference"))
NVCC = "/usr/local/cuda/bin/nvcc"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(with_reference: bool = True) -> dict:
    out = {}
    steps = []
    lib = ORACLE / "liboracle.so"
    src = ORACLE / "oracle.cpp"
    if _stale(lib, [src]):
        steps.append(["g++", "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                      str(src), "-o", str(lib)])
    out["oracle"] = str(lib)
    rr = ORACLE / "liborc_refrun.so"
    rsrc = ORACLE / "ref_runner.cu"
    if Path(NVCC).exists() and _stale(rr, [rsrc]):
        steps.append([NVCC] + ARCH + ["-O2", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-shared",
                                      str(rsrc), "-o", str(rr)])
    out["refrun"] = str(rr)
    if with_reference and (REFERENCE / "FunctionOnGPU.cu").exists():
        REF_OUT.mkdir(exist_ok=True)
        cubin = REF_OUT / "ref_kernels.cubin"
        shim = ORACLE / "ref_shim"
        deps = [REFERENCE / n for n in ("FunctionOnGPU.cu", "FunctionOnGPU.cuh", "MrcFileIOBaseFunction.h",
                                        "MrcFileIO.h", "ReadAndInitialOptions.h", "MpiBigData.h")]
        if _stale(cubin, deps + [shim / "mpi.h"]):
            # CHECK is used but never defined in FunctionOnGPU.cu:216-217; map it to the
            # file's own checkCudaErrors.  mpi.h: declarations only (no MPI code runs).
            steps.append([NVCC] + ARCH + ["-cubin", "-DCHECK=checkCudaErrors", "-I", str(shim), "-I",
                                          str(REFERENCE), str(REFERENCE / "FunctionOnGPU.cu"), "-o", str(cubin)])
        out["ref_cubin"] = str(cubin)
        gold = REF_OUT / "ref_golden"
        gsrc = [ORACLE / "ref_golden.cpp"] + [REFERENCE / n for n in ("MrcFileIO.cpp", "MrcFileIOBaseFunction.cpp",
                                                                        "ReadAndInitialOptions.cpp")]
        if platform.machine() in ("x86_64", "AMD64") and _stale(gold, gsrc + deps + [ORACLE / "ref_shim_host" / "cuda_runtime.h"]):
            # char is signed on x86-64, which the reference's getopt loop needs
            # (ReadAndInitialOptions.cpp:142-143); the generator is built here only.
            steps.append(["g++", "-O0", "-std=c++11", "-w", "-fsigned-char", "-I", str(REFERENCE), "-I",
                          str(ORACLE / "ref_shim_host")] + [str(s) for s in gsrc] + ["-o", str(gold)])
        out["ref_golden"] = str(gold)
    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        for f in [ex.submit(_run, c) for c in steps]:
            f.result()
    return out


if __name__ == "__main__":
    print(build())
