"""Builds libhorender.so in place (this directory) for sm_103a.

Every translation unit is compiled in parallel with nvcc (one -gencode,
sm_103a only), then linked into one shared library with the CUDA runtime
linked statically, so the library needs nothing but the driver at run time.

    python test-_gb300/build.py            # build if sources changed
    python test-_gb300/build.py --force    # rebuild everything
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = HERE / "csrc"
OBJ = HERE / "_build"
LIB = HERE / "libhorender.so"
CLI_SRC = HERE / "cli" / "horender_cli.cpp"
CLI = HERE / "horender_cli"
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-O2", "-I", str(ROOT / "include"),
          "-I", str(CSRC)]
CU_FLAGS = ARCH + COMMON + ["--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]
# per-file extras: the primitive pass rounds every operation on its own, as
# the reference's FP32 host code does (its start searches branch on exact
# values); the host scene numerics fuse no multiply-adds, so a seeded scene
# has the same bits on x86-64 and aarch64 hosts (as far as their libm agrees)
FILE_FLAGS = {"ho_prim.cu": ["--fmad=false"], "ho_scene.cpp": ["-Xcompiler", "-ffp-contract=off"]}


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h")))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    hdrs = headers()
    procs = []
    objs = []
    for src in sources():
        obj = OBJ / (src.name + ".o")
        objs.append(obj)
        if not force and not _stale(obj, [src] + hdrs):
            continue
        if src.suffix == ".cu":
            cmd = [NVCC] + CU_FLAGS + FILE_FLAGS.get(src.name, []) + ["-c", str(src), "-o", str(obj)]
        else:
            cmd = [NVCC] + ARCH + COMMON + FILE_FLAGS.get(src.name, []) + ["-x", "c++", "-c", str(src), "-o", str(obj)]
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((src, out))
        elif verbose and out.strip():
            print(f"--- {src.name}\n{out}")
    if failed:
        msg = "\n".join(f"--- {s.name}\n{o}" for s, o in failed)
        raise RuntimeError(f"nvcc failed:\n{msg}")
    if force or _stale(LIB, objs):
        cmd = [NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", str(LIB)] + [str(o) for o in objs] + ["-lpthread"]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}")
    # the command-line renderer, linked against the library beside it
    if force or _stale(CLI, [CLI_SRC, LIB, ROOT / "include" / "horender.hpp", ROOT / "include" / "horender.h"]):
        cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-I", str(ROOT / "include"), str(CLI_SRC),
               "-L", str(HERE), "-lhorender", "-Wl,-rpath,$ORIGIN", "-o", str(CLI)]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed:\n{r.stdout}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
