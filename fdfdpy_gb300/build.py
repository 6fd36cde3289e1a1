"""Build the engine's shared library ``libfdfd_gb300.so`` in-tree.

The CUDA sources are compiled for sm_103a only (one ``-gencode``), each
translation unit in its own nvcc process, then linked with ``nvcc -shared``.
No cmake, no torch extension machinery: the library exposes a plain C ABI
(``include/fdfd_gb300.h``) and the Python host binds it with ctypes.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libfdfd_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the FDFD engine needs the CUDA toolkit to build")


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _flags(src: Path):
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-I", str(CSRC), "-I", str(PKG.parent / "include")]
    if src.suffix == ".cu":
        return common + ARCH + ["-lineinfo", "--expt-relaxed-constexpr"]
    return common


def _up_to_date(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return False
    deps = [src] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [PKG.parent / "include" / "fdfd_gb300.h"]
    t = obj.stat().st_mtime
    return all(d.stat().st_mtime <= t for d in deps if d.exists())


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compile every source under csrc/ and link libfdfd_gb300.so."""
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    srcs = _sources()
    objs = [BUILD / (s.name + ".o") for s in srcs]

    def compile_one(args):
        src, obj = args
        if not force and _up_to_date(obj, src):
            return None
        cmd = [nvcc, "-c", str(src), "-o", str(obj)] + _flags(src)
        if verbose:
            print(" ".join(cmd), flush=True)
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
        return res.stderr

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        for out in ex.map(compile_one, zip(srcs, objs)):
            if out and verbose:
                print(out, file=sys.stderr)
    relink = force or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs)
    if relink:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, "-shared", "-o", str(tmp)] + [str(o) for o in objs] + ARCH + [
            "-cudart", "shared", "-Xlinker", "-rpath=/usr/local/cuda/lib64"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
