"""In-tree build of the native library ``libsharpray_gb300.so`` (CUDA kernels for sm_103a + the
C-ABI host code).  Translation units compile in parallel; the whole build takes well under a minute.

Run ``python -m sharpray_gb300.build`` or call :func:`build_library`.
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
LIB = PKG / "libsharpray_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_SOURCES = ["sr_render.cu", "sr_wavefront.cu", "sr_wave_adjoint.cu", "sr_wave_trace.cu", "sr_compose.cu",
                "sr_bvh_build.cu", "sr_overlay.cu", "sr_adjoint.cu"]
HOST_SOURCES = ["sr_host.cpp", "sr_geometry.cpp", "sr_ingest.cpp", "sr_image.cpp"]


def cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed ({proc.returncode}):\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def build_library(verbose: bool = False, ptxas_info: bool = False, defines: tuple = (), out: Path | None = None,
                  build_dir: Path | None = None) -> Path:
    """Compile every translation unit and link the shared library.  Returns its path.

    `defines` are extra -D tuning macros (SR_REFILL, SR_TRACE_MIN_BLOCKS, SR_LEAF_LOOP); `out` and
    `build_dir` redirect the outputs (defaults: the in-tree library)."""
    cuda = cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    bdir = build_dir or BUILD
    lib = out or LIB
    bdir.mkdir(parents=True, exist_ok=True)
    inc = [f"-I{ROOT / 'include'}", f"-I{CSRC}", f"-I{cuda / 'include'}"] + [f"-D{d}" for d in defines]
    jobs = []
    for src in CUDA_SOURCES:
        obj = bdir / (src + ".o")
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
               "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", *inc, "-c", str(CSRC / src), "-o", str(obj)]
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((cmd, obj))
    for src in HOST_SOURCES:
        obj = bdir / (src + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fvisibility=hidden",
               "-Wall", *inc, "-c", str(CSRC / src), "-o", str(obj)]
        jobs.append((cmd, obj))
    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        futures = [ex.submit(_run, cmd) for cmd, _ in jobs]
        for f in futures:
            f.result()
    tmp = lib.with_suffix(".so.tmp")
    link = [nvcc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-cudart", "static", *[str(o) for _, o in jobs],
            "-o", str(tmp)]
    _run(link)
    os.replace(tmp, lib)
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build_library(verbose=True, ptxas_info="--ptxas" in sys.argv)
