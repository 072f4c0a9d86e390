"""Build recipe for the reference's own C++ core (test infrastructure only).

Compiles the reference's sources where they lie (``src/qhmat/core.cpp``,
``src/qhmat/io.cpp`` and, when pybind11 is importable, ``src/qhmat/bindings.cpp``)
with g++ directly -- no CMake, no copy of any reference source -- and writes
only into ``oracle/_ref/``:

* ``oracle/_ref/libqhmat_ref.so``: the reference core plus ``oracle/ref_shim.cpp``
  (a C ABI over ``HMatrix::load/matmul/reconstruct``), loaded with ctypes by the
  tests and by ``bench.py``'s CPU-baseline leg;
* ``oracle/_ref/qhmat_core/_core<EXT_SUFFIX>``: the reference's pybind11 module,
  used by ``tests/golden/make_golden.py`` to build fixtures with the reference's
  own ``HMatrix.from_dense``.

The reference tree is only present in the build container; where it is
absent this recipe does nothing and reports why.
"""

from __future__ import annotations

import os
import subprocess
import sys
import sysconfig
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
DEFAULT_REFERENCE = Path(os.environ.get("QHMAT_REFERENCE", "/root/reference"))


def _run(cmd: list[str]) -> None:
    subprocess.run(cmd, check=True)


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build(reference: Path = DEFAULT_REFERENCE, verbose: bool = False) -> bool:
    """Compile the reference core into ``oracle/_ref``; return False if absent."""
    src = reference / "src"
    core = src / "qhmat" / "core.cpp"
    io = src / "qhmat" / "io.cpp"
    if not core.exists() or not io.exists():
        if verbose:
            print(f"reference sources not found under {reference}; oracle/_ref not built")
        return False
    OUT.mkdir(parents=True, exist_ok=True)
    flags = ["-O2", "-std=c++17", "-fPIC", "-shared", f"-I{src}"]

    lib = OUT / "libqhmat_ref.so"
    shim = HERE / "ref_shim.cpp"
    if _stale(lib, [core, io, shim]):
        _run(["g++", *flags, str(shim), str(core), str(io), "-o", str(lib)])

    try:
        import pybind11  # noqa: F401  (only in the build container)
    except ImportError:
        return True
    import pybind11

    bindings = src / "qhmat" / "bindings.cpp"
    pkg = OUT / "qhmat_core"
    pkg.mkdir(exist_ok=True)
    ext = pkg / ("_core" + sysconfig.get_config_var("EXT_SUFFIX"))
    if _stale(ext, [core, io, bindings]):
        inc = [f"-I{pybind11.get_include()}", f"-I{sysconfig.get_paths()['include']}"]
        _run(["g++", *flags, *inc, "-fvisibility=hidden", str(bindings), str(core),
              str(io), "-o", str(ext)])
    return True


def import_reference_qhmat(reference: Path = DEFAULT_REFERENCE):
    """Import the reference's ``qhmat`` package with the extension built above."""
    import importlib.util

    if "qhmat" in sys.modules:
        return sys.modules["qhmat"]
    if not build(reference):
        raise RuntimeError(f"reference sources not found under {reference}")
    ext = next((OUT / "qhmat_core").glob("_core*"))
    spec = importlib.util.spec_from_file_location("qhmat._core", ext)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    sys.modules["qhmat._core"] = mod
    sys.path.insert(0, str(reference / "python"))
    import qhmat

    return qhmat


if __name__ == "__main__":
    ok = build(verbose=True)
    print("built" if ok else "skipped")
