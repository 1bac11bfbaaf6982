"""Build recipe of libpysit_gb300.so (sm_103a only) and of the test-only oracle.

``python -m pysit_gb300.build`` compiles every ``csrc/*.cu`` translation unit in
parallel with nvcc (``-gencode arch=compute_103a,code=sm_103a``) and links the
shared library in-tree (``pysit_gb300/libpysit_gb300.so``).  Object files go
to ``pysit_gb300/_build/``.  Nothing is installed into site-packages.

"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpysit_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pysit_gb300")


def _defines() -> list[str]:
    """Extra -D flags of every translation unit (none: the kernels' macros keep their defaults).
    The object directory records them, so a change rebuilds every object."""
    return []


def _flags(verbose_ptxas: bool = False) -> list[str]:
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")] + _defines()
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _compile(src: str, verbose_ptxas: bool) -> tuple[str, str]:
    obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".cuh")]
    deps.append(os.path.join(ROOT, "include", "pysit_gb300.h"))
    if (not verbose_ptxas and os.path.exists(obj)
            and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps)):
        return obj, ""
    cmd = [_nvcc()] + _flags(verbose_ptxas) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stdout + r.stderr


def build(verbose_ptxas: bool = False, jobs: int | None = None) -> str:
    """Compile and link the CUDA library; returns its path."""
    os.makedirs(OBJ, exist_ok=True)
    stamp = os.path.join(OBJ, "defines.txt")
    want = " ".join(_defines())
    have = ""
    if os.path.exists(stamp):
        with open(stamp) as fh:
            have = fh.read()
    if want != have:  # other macros: every object is stale
        for f in os.listdir(OBJ):
            if f.endswith(".o"):
                os.remove(os.path.join(OBJ, f))
        with open(stamp, "w") as fh:
            fh.write(want)
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    logs = []
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = []
        for obj, log in ex.map(lambda s: _compile(s, verbose_ptxas), srcs):
            objs.append(obj)
            if log:
                logs.append(log)
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp"
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose_ptxas:
        sys.stdout.write("\n".join(logs))
    return LIB


def build_oracle() -> None:
    """Compile the test-only CPU oracle (and, where the reference tree exists, the reference)."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "all"], check=True)


if __name__ == "__main__":
    print(build(verbose_ptxas="-v" in sys.argv))
