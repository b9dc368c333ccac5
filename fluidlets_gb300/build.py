"""Build libfluidlets_gb300.so in-tree with nvcc (sm_103a only).

    python -m fluidlets_gb300.build        # or __graft_entry__.build()

Each translation unit in csrc/ is compiled in parallel to an object file,
then linked into fluidlets_gb300/_build/libfluidlets_gb300.so.  The library
links only the CUDA runtime (and cuBLAS for nothing: it does not link it).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT_DIR = HERE / "_build"
LIB_NAME = "libfluidlets_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "--expt-relaxed-constexpr", "-I", str(HERE.parent / "include")]
# translation units whose FP32 code wants flush-to-zero (the far-field kernels
# use the approximate MUFU instructions with .ftz anyway)
FTZ = {"sum.cu"}


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return exe


def sources():
    return sorted(CSRC.glob("*.cu"))


def _compile(src: Path, obj: Path, verbose: bool) -> None:
    cmd = [nvcc(), *ARCH, *COMMON, "-c", str(src), "-o", str(obj)]
    if src.name in FTZ:
        cmd.insert(1, "-ftz=true")
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")


def lib_path() -> Path:
    return OUT_DIR / LIB_NAME


def needs_build() -> bool:
    lib = lib_path()
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = list(CSRC.glob("*")) + [HERE.parent / "include" / "fluidlets_gb300.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> Path:
    if not force and not needs_build():
        return lib_path()
    OUT_DIR.mkdir(exist_ok=True)
    srcs = sources()
    objs = [OUT_DIR / (s.stem + ".o") for s in srcs]
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        list(ex.map(lambda so: _compile(so[0], so[1], verbose), zip(srcs, objs)))
    tmp = OUT_DIR / f"{LIB_NAME}.{os.getpid()}"
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path())
    return lib_path()


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
