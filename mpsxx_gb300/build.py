"""Build libmpsxx_gb300.so in-tree with nvcc for sm_103a (no cmake)."""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
LIBDIR = HERE / "lib"
LIBNAME = "libmpsxx_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def sources():
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def build(verbose: bool = False, force: bool = False) -> Path:
    LIBDIR.mkdir(exist_ok=True)
    objdir = LIBDIR / "obj"
    objdir.mkdir(exist_ok=True)
    out = LIBDIR / LIBNAME
    srcs = sources()
    headers = list(CSRC.glob("*.hpp")) + list((HERE.parent / "include").glob("*.h"))
    newest_dep = max(p.stat().st_mtime for p in srcs + headers)
    common = [nvcc(), ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "-I", str(CSRC), "-I", str(HERE.parent / "include")]

    def compile_one(src: Path):
        obj = objdir / (src.name + ".o")
        if not force and obj.exists() and obj.stat().st_mtime >= newest_dep:
            return obj
        cmd = common + ["-c", str(src), "-o", str(obj)]
        if src.suffix == ".cpp":
            cmd = common + ["-x", "cu", "-c", str(src), "-o", str(obj)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src.name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    if force or not out.exists() or out.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        cmd = [nvcc(), ARCH, "-shared", "-o", str(out)] + [str(o) for o in objs] + ["-lcusolver", "-lcublas", "-lcudart", "-Xlinker", "-rpath,/usr/local/cuda/lib64"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return out


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
