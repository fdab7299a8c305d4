"""Build the CUDA library in-tree with nvcc (sm_103a only).

    python -m fastode_gb300.build        # or fastode_gb300.build.build()

The library is a plain C-ABI shared object (include/fastode_gb300.h), loaded
with ctypes; it carries no PyTorch types. Translation units compile in
parallel (nvcc --threads) with a single -gencode, so the build takes seconds.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIBDIR = PKG / "_lib"
LIBNAME = "libfastode_gb300.so"
SOURCES = ["integrator.cu", "adjoint.cu", "abi.cu", "utility.cu", "scoring.cu", "static_scratch.cu", "symbolic.cpp",
           "codegen.cpp", "jit.cpp", "embed.cpp"]
# the integrator of the generated variant, compiled as relocatable device code
# and embedded in the library (embed.cpp), where each plan links it with its
# mechanism's generated code
RDC_SOURCE = "generated.cu"
RDC_NAME = "generated_rdc.cubin"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc_path() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build fastode_gb300")


def library_path() -> Path:
    return LIBDIR / LIBNAME


def _stale(target: Path) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    deps = [CSRC / s for s in SOURCES + [RDC_SOURCE]] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh"))
    deps.append(ROOT / "include" / "fastode_gb300.h")
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(force: bool = False, verbose: bool = False) -> Path:
    target = library_path()
    if not force and not _stale(target):
        return target
    LIBDIR.mkdir(exist_ok=True)
    tmp = target.with_suffix(".so.tmp%d" % os.getpid())
    rdc = LIBDIR / RDC_NAME
    rdc_tmp = rdc.with_suffix(".cubin.tmp%d" % os.getpid())
    steps = [
        [nvcc_path(), "-cubin", "-rdc=true", *ARCH, "-O3", "-lineinfo", "-std=c++17", f"-I{ROOT / 'include'}",
         str(CSRC / RDC_SOURCE), "-o", str(rdc_tmp)],
        [nvcc_path(), "-shared", "-Xcompiler", "-fPIC", *ARCH, "-O3", "-lineinfo", "-std=c++17",
         "--threads", "0", f"-I{ROOT / 'include'}", f'-DFO_GENERATED_RDC="{rdc}"',
         *[str(CSRC / s) for s in SOURCES], "-ldl", "-o", str(tmp)],
    ]
    for i, cmd in enumerate(steps):
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + r.stdout + r.stderr)
        if verbose:
            print(r.stdout + r.stderr, file=sys.stderr)
        if i == 0:
            os.replace(rdc_tmp, rdc)
    os.replace(tmp, target)
    return target


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
