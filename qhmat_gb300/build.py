"""Build recipe for the CUDA library (sm_103a only).

Compiles ``csrc/*.cu`` and ``csrc/*.cpp`` with nvcc into the in-tree shared
library ``qhmat_gb300/libqhmat_gb300.so`` (the C ABI declared in
``include/qhmat_gb300.h``).  Translation units compile in parallel; the CUDA
runtime is linked statically so the library loads beside any torch build.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libqhmat_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build qhmat_gb300")


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.hpp")) + sorted((ROOT / "include").glob("*.h"))


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compile (if stale) and return the path of libqhmat_gb300.so."""
    srcs = _sources()
    deps = srcs + _headers() + [Path(__file__)]
    newest = max(p.stat().st_mtime for p in deps)
    if not force and LIB.exists() and LIB.stat().st_mtime >= newest:
        return LIB
    OBJ.mkdir(exist_ok=True)
    cc = nvcc()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
              f"-I{ROOT / 'include'}", f"-I{CSRC}"]

    def compile_one(src: Path) -> Path:
        obj = OBJ / (src.name + ".o")
        cmd = [cc, *common, "-c", str(src), "-o", str(obj)]
        if src.suffix == ".cu":
            cmd[1:1] = [*ARCH, "-lineinfo", "-Xptxas", "-v" if verbose else "-O3"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"compiling {src.name} failed:\n{res.stdout}{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 1))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB.with_suffix(f".{os.getpid()}.tmp")
    res = subprocess.run([cc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static"],
                         capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"linking libqhmat_gb300.so failed:\n{res.stdout}{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
