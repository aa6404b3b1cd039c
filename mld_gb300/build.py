"""Build libmld_gpu.so (sm_103a) in-tree with nvcc; no cmake, one -gencode, parallel TUs."""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libmld_gpu.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["api.cu", "bispectrum.cu", "neighbours.cu", "fit.cu", "quad.cu", "solve.cu", "gram_tc.cu", "kernel_rows.cu", "serve.cu", "noalloc.cu", "precond32.cu", "eval.cu", "krr_tc.cu", "sketch.cu", "rows.cu",
           "bso4_tables.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), *NVCC_FLAGS, *extra, "-x", "c++", "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


STAMP = OUT + ".srchash"


def source_hash(extra: list[str]) -> str:
    """SHA-256 over the sources, the public header, the compiler flags and nvcc's version, so a
    library built elsewhere (another machine's copy of the tree) is never mistaken for current."""
    h = hashlib.sha256()
    deps = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)) + [os.path.join(HERE, "..", "include", "mld_gpu.h")]
    for d in deps:
        if os.path.isfile(d):
            h.update(os.path.basename(d).encode())
            with open(d, "rb") as fh:
                h.update(fh.read())
    h.update(" ".join(ARCH + NVCC_FLAGS[:-2] + list(extra)).encode())
    h.update(platform.machine().encode())
    try:
        h.update(subprocess.run([nvcc(), "--version"], capture_output=True, text=True).stdout.encode())
    except Exception:  # pragma: no cover - nvcc missing: build() fails later with its own message
        pass
    return h.hexdigest()


def up_to_date(extra: list[str] | None = None) -> bool:
    if not (os.path.exists(OUT) and os.path.exists(STAMP)):
        return False
    with open(STAMP) as fh:
        return fh.read().strip() == source_hash(list(extra or []))


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    if not force and up_to_date(extra):
        return OUT
    os.makedirs(BUILD, exist_ok=True)
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = OUT + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    with open(STAMP, "w") as fh:
        fh.write(source_hash(extra) + "\n")
    if verbose:
        print("built", OUT)
    return OUT


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True,
          extra=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else None)
