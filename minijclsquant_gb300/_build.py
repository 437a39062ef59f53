"""Compile libkpm (the sm_103a CUDA kernels behind include/kpm.h) in-tree.

Each ``csrc/*.cu`` is compiled in parallel to an object with
``-gencode arch=compute_103a,code=sm_103a``; the objects are linked into
``minijclsquant_gb300/_build/libkpm.so`` (static CUDA runtime, so the library
only needs the driver).  Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG_DIR, "csrc")
BUILD_DIR = os.path.join(PKG_DIR, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libkpm.so")
INCLUDE_DIR = os.path.join(os.path.dirname(PKG_DIR), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def _nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers_digest() -> str:
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE_DIR):
        for f in sorted(os.listdir(d)):
            if f.endswith((".cuh", ".h")):
                with open(os.path.join(d, f), "rb") as fh:
                    h.update(f.encode())
                    h.update(fh.read())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    return h.hexdigest()[:16]


def _obj_for(src: str, digest: str) -> str:
    with open(src, "rb") as fh:
        sh = hashlib.sha256(fh.read()).hexdigest()[:16]
    base = os.path.splitext(os.path.basename(src))[0]
    return os.path.join(BUILD_DIR, "%s.%s.%s.o" % (base, sh, digest))


def _compile(src: str, obj: str) -> str:
    tmp = obj + ".tmp.o"
    cmd = [_nvcc()] + ARCH + NVCC_FLAGS + ["-I", INCLUDE_DIR, "-c", src, "-o", tmp]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s" % (os.path.basename(src), r.stdout))
    os.replace(tmp, obj)
    return r.stdout


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Build (or reuse) libkpm.so and return its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    digest = _headers_digest()
    srcs = sources()
    objs = [_obj_for(s, digest) for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if not os.path.exists(o)]
    if todo:
        jobs = jobs or min(len(todo), max(1, os.cpu_count() or 1))
        with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
            for out in ex.map(lambda so: _compile(*so), todo):
                if verbose and out.strip():
                    sys.stderr.write(out)
    stamp = os.path.join(BUILD_DIR, "libkpm.objs")
    want = "\n".join(objs)
    have = open(stamp).read() if os.path.exists(stamp) else ""
    if have != want or not os.path.exists(LIB_PATH):
        tmp = LIB_PATH + ".tmp"
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs
        subprocess.run(cmd, check=True)
        os.replace(tmp, LIB_PATH)
        with open(stamp, "w") as fh:
            fh.write(want)
    # drop stale objects
    keep = set(objs)
    for f in os.listdir(BUILD_DIR):
        p = os.path.join(BUILD_DIR, f)
        if f.endswith(".o") and p not in keep:
            os.remove(p)
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
