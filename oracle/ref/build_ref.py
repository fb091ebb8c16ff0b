"""Build poutre2's own hot-path sources into oracle/_ref/libpoutre_ref.so.

TEST INFRASTRUCTURE ONLY (checker + CPU baseline).  Recipe:

1. ``stage``: when the poutre2 tree is given (the ``root`` argument, else the environment
   variable ``POUTRE2_REFERENCE``), copy the headers under ``include/poutre`` and the ``.cpp`` files
   of the modules on the path (base, pixel_processing, structuring_element,
   low_level_morpho, geodesy) and of label into ``oracle/_ref/src``.  ``oracle/_ref`` is git-ignored,
   so no reference source enters the repository; the staged copy only lets the same
   recipe run on a machine that does not mount the tree (the aarch64 GPU host).
2. ``compile``: ``g++ -std=c++23 -O3`` on the staged sources plus ``ref_harness.cpp``,
   with project-written stand-ins for the two absent third-party headers
   (``shim/xsimd`` for xsimd 14.2.0, ``shim/spdlog`` for spdlog 1.17.0) and the forced
   includes the sources rely on transitively (``cstring``, ``mutex``, ``cmath``).
   The ISA is the host's: ``-mavx2`` on x86-64 (poutre2's default), NEON on aarch64.
   The reference's own CMake build is not used.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
STAGE = os.path.join(OUT, "src")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libpoutre_ref.so")
MODULES = ["base", "pixel_processing", "structuring_element", "low_level_morpho", "geodesy", "label"]


def reference_root(root: str | None = None) -> str | None:
    """The poutre2 source tree: `root`, else $POUTRE2_REFERENCE, else None (no default)."""
    return root or os.environ.get("POUTRE2_REFERENCE") or None


def has_tree(root: str | None) -> bool:
    return bool(root) and os.path.isdir(os.path.join(root, "include", "poutre"))


def stage(root: str | None = None) -> bool:
    root = reference_root(root)
    if not has_tree(root):
        return os.path.isdir(STAGE)
    if os.path.isdir(STAGE):
        shutil.rmtree(STAGE)
    shutil.copytree(os.path.join(root, "include", "poutre"), os.path.join(STAGE, "include", "poutre"))
    for m in MODULES:
        dst = os.path.join(STAGE, "src", m)
        os.makedirs(dst, exist_ok=True)
        for f in glob.glob(os.path.join(root, "src", m, "*.cpp")):
            shutil.copy2(f, dst)
    return True


def _flags():
    f = ["-std=c++23", "-O3", "-DNDEBUG", "-fPIC", "-w",
         "-I", os.path.join(STAGE, "include"), "-I", os.path.join(HERE, "shim"),
         "-include", "cstring", "-include", "mutex", "-include", "cmath"]
    if platform.machine() in ("x86_64", "AMD64"):
        f.append("-mavx2")
    return f


def _compile_one(src: str) -> str:
    rel = os.path.relpath(src, STAGE) if src.startswith(STAGE) else os.path.basename(src)
    obj = os.path.join(OBJ, rel.replace(os.sep, "_") + ".o")
    if not os.path.exists(obj) or os.path.getmtime(obj) < os.path.getmtime(src):
        flags = _flags()
        if os.path.basename(src) == "compare.cpp":
            # ~100 s at -O3 (eight overloads x five pixel types); at -O1 it builds in ~40 s.
            # Only the pointwise CompareImage step of the binary h-maxima baseline uses it.
            flags = [f if f != "-O3" else "-O1" for f in flags]
        subprocess.check_call(["g++"] + flags + ["-c", src, "-o", obj])
    return obj


def compile_lib(jobs: int | None = None) -> str:
    if not os.path.isdir(STAGE):
        raise RuntimeError("poutre2 sources are not staged (oracle/_ref/src missing)")
    os.makedirs(OBJ, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(STAGE, "src", "*", "*.cpp")), key=lambda s: "compare.cpp" not in s)
    srcs += [os.path.join(HERE, "ref_harness.cpp")]
    jobs = jobs or max(1, min(len(srcs), os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(_compile_one, srcs))
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["g++", "-shared", "-o", tmp] + objs)
    os.replace(tmp, LIB)
    return LIB


def build(root: str | None = None) -> str | None:
    """Stage (when the tree is given) and compile; returns the library path or None."""
    if not stage(root):
        return None
    return compile_lib()


if __name__ == "__main__":
    p = build(sys.argv[1] if len(sys.argv) > 1 else None)
    print(p or "poutre2 sources unavailable: oracle/_ref not built")
    sys.exit(0)
