"""Builds the GB300 extension in-tree.

Outputs (git-ignored, rebuilt on every machine):
  pattenmatching_sharedmemory_gb300/lib/libpm_gb300.so     the C-ABI library
  pattenmatching_sharedmemory_gb300/lib/patternmatching_gb300  the CLI
Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a); host C++ with g++ (-fopenmp,
-ffp-contract=off so the seeded input generators give identical graphs on
x86 and aarch64).  Translation units compile in parallel; a content stamp
skips the build when nothing changed.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "lib"
OBJ_DIR = PKG / "_build"
LIB = LIB_DIR / "libpm_gb300.so"
CLI = LIB_DIR / "patternmatching_gb300"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["kernels_lcc.cu", "kernels_walk.cu"]
CC_SOURCES = ["totem_io.cc", "constraints.cc", "effectiveness.cc", "walk_compile.cc", "generators.cc", "engine.cc",
              "server.cc",
              "fused_batch.cc", "autotune.cc", "capi.cc"]


def _sources() -> tuple[list[Path], list[Path]]:
    cu = [CSRC / s for s in CU_SOURCES]
    cc = [CSRC / s for s in CC_SOURCES]
    return cu, cc


def _stamp() -> str:
    h = hashlib.sha256()
    for p in sorted(CSRC.glob("*")) + sorted((ROOT / "include").glob("*.h")) + [Path(__file__)]:
        if p.is_file():
            h.update(p.name.encode())
            h.update(p.read_bytes())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles the extension (if sources changed) and returns the .so path."""
    stamp_file = OBJ_DIR / "stamp"
    stamp = _stamp()
    if not force and LIB.exists() and CLI.exists() and stamp_file.exists() and stamp_file.read_text() == stamp:
        return LIB
    if shutil.which(NVCC) is None and not Path(NVCC).exists():
        raise RuntimeError(f"nvcc not found at {NVCC}; the GB300 extension cannot be built")
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    cu, cc = _sources()
    inc = [f"-I{CSRC}", f"-I{ROOT / 'include'}", f"-I{CUDA_HOME / 'include'}"]
    jobs = []
    for src in cu:
        obj = OBJ_DIR / (src.stem + ".cu.o")
        jobs.append([NVCC, "-std=c++17", "-O3", *ARCH, "-lineinfo", "-Xcompiler", "-fPIC", *inc, "-c", str(src),
                     "-o", str(obj)])
    for src in cc:
        obj = OBJ_DIR / (src.stem + ".o")
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", *inc, "-c", str(src),
                     "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=max(2, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(_run, jobs))
    objs = [str(OBJ_DIR / (s.stem + ".cu.o")) for s in cu] + [str(OBJ_DIR / (s.stem + ".o")) for s in cc]
    cudalib = CUDA_HOME / "lib64"
    if not cudalib.exists():
        cudalib = CUDA_HOME / "lib"
    tmp = LIB.with_suffix(".so.tmp")
    _run(["g++", "-shared", "-o", str(tmp), *objs, f"-L{cudalib}", "-lcudart_static", "-ldl", "-lrt", "-lpthread",
          "-fopenmp"])
    os.replace(tmp, LIB)
    cli_obj = OBJ_DIR / "cli.o"
    _run(["g++", "-std=c++17", "-O2", *inc, "-c", str(CSRC / "cli.cc"), "-o", str(cli_obj)])
    _run(["g++", "-o", str(CLI), str(cli_obj), str(LIB), f"-Wl,-rpath,{LIB_DIR}"])
    stamp_file.write_text(stamp)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
