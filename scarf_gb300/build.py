"""Build recipe of the scarf_gb300 CUDA library (sm_103a).

Every ``csrc/*.cu`` (and host-only ``csrc/*.cpp``) is compiled by nvcc in parallel into ``_build/`` and
linked into ``_build/libscarfgpu.so``. The library is loaded in-tree by
``scarf_gb300._lib``; nothing is installed.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
OUT = HERE / "_build"
LIB = OUT / "libscarfgpu.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def cuda_lib_dir() -> str:
    root = Path(nvcc()).resolve().parent.parent
    for d in (root / "lib64", root / "lib", root / "targets" / "sbsa-linux" / "lib",
              root / "targets" / "x86_64-linux" / "lib"):
        if (d / "libcudart.so").exists() or (d / "libcusolver.so").exists():
            return str(d)
    return str(root / "lib64")


def _flags(verbose_ptx: bool = False):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                "-I", str(HERE.parent / "include")]
    if verbose_ptx:
        f += ["-Xptxas", "-v"]
    return f


def _compile(src: Path, verbose_ptx: bool) -> tuple[Path, str]:
    obj = OUT / (src.stem + ".o")
    cmd = [nvcc(), "-c", str(src), "-o", str(obj)] + _flags(verbose_ptx)
    if src.suffix == ".cpp":  # host code: the same arithmetic on x86 and Arm hosts
        cmd += ["-Xcompiler", "-ffp-contract=off"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def up_to_date() -> bool:
    if not LIB.exists():
        return False
    t = LIB.stat().st_mtime
    deps = (list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")) + list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h"))
            + list((HERE.parent / "include").glob("*.h")))
    deps.append(Path(__file__))
    return all(p.stat().st_mtime <= t for p in deps)


def build(force: bool = False, verbose_ptx: bool = False, quiet: bool = True) -> Path:
    if not force and up_to_date():
        return LIB
    OUT.mkdir(exist_ok=True)
    srcs = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    logs = []
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        for obj, log in ex.map(lambda s: _compile(s, verbose_ptx), srcs):
            logs.append((obj, log))
    objs = [str(o) for o, _ in logs]
    tmp = OUT / "libscarfgpu.so.tmp"
    cmd = [nvcc(), "-shared", "-o", str(tmp)] + objs + ARCH + [
        "-L", cuda_lib_dir(), "-lcusolver", "-lcublas", "-lcudart", "-Xlinker", "-rpath=" + cuda_lib_dir()]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose_ptx or not quiet:
        for obj, log in logs:
            sys.stderr.write(f"== {obj.name}\n{log}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptx="-v" in sys.argv, quiet=False)
    print(LIB)
