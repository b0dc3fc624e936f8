"""In-tree build of the sm_103a device backend library ``librstsr_cuda.so``.

Every ``csrc/*.cu`` is compiled by nvcc for ``sm_103a`` only and every
``csrc/*.cpp`` by the host compiler, in parallel, into ``_build/``; the objects
are linked into ``_build/librstsr_cuda.so`` against the shared CUDA runtime.
An object is rebuilt when its source or any header is newer than it.
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
INCLUDE = ROOT / "include"
BUILD = PKG / "_build"
LIB = BUILD / "librstsr_cuda.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-fvisibility=hidden",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", "-Wall"]


def _cuda_home() -> Path:
    env = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if env:
        return Path(env)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path("/usr/local/cuda")


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.hpp")) + list(INCLUDE.glob("*.h")))


def _stale(obj: Path, src: Path, hdr_mtime: float) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return t < src.stat().st_mtime or t < hdr_mtime


def _run(cmd: list[str]) -> tuple[list[str], int, str]:
    p = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, p.returncode, p.stdout + p.stderr


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile and link the library; returns its path. Raises on failure."""
    cuda = _cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    cxx = os.environ.get("CXX", "g++")
    BUILD.mkdir(exist_ok=True)
    hdr_mtime = max((h.stat().st_mtime for h in _headers()), default=0.0)
    incs = [f"-I{INCLUDE}", f"-I{CSRC}"]
    cmds = []
    objs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = BUILD / (src.stem + ".cu.o")
        objs.append(obj)
        if _stale(obj, src, hdr_mtime):
            cmds.append([nvcc, *NVCC_FLAGS, *incs, "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = BUILD / (src.stem + ".cpp.o")
        objs.append(obj)
        if _stale(obj, src, hdr_mtime):
            cmds.append([cxx, *CXX_FLAGS, *incs, f"-I{cuda / 'include'}", "-c", str(src), "-o", str(obj)])
    jobs = jobs or max(1, min(len(cmds), os.cpu_count() or 4))
    errors = []
    if cmds:
        with ThreadPoolExecutor(max_workers=jobs) as ex:
            for cmd, rc, out in ex.map(_run, cmds):
                if verbose or rc != 0:
                    print(" ".join(cmd[-3:]), file=sys.stderr)
                    if out.strip():
                        print(out, file=sys.stderr)
                if rc != 0:
                    errors.append(cmd[-3])
    if errors:
        raise RuntimeError(f"compilation failed for: {', '.join(errors)}")
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        link = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        cmd, rc, out = _run(link)
        if rc != 0:
            print(out, file=sys.stderr)
            raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
