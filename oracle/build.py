"""Build recipe for the oracle -- TEST INFRASTRUCTURE ONLY.

Two artefacts, both used only by ``tests/``, ``__graft_entry__.smoke()`` and the
CPU legs of ``bench.py``:

* ``oracle/_build/libkpm_oracle.so`` -- the plain-C restatement in
  ``kpm_oracle.c`` (gcc, OpenMP, portable flags: builds on x86_64 and aarch64).
* ``oracle/_ref/`` -- jclsquant's own Cython kernels (``blas_funs.pyx``,
  ``Extra_funs.pyx``), translated by Cython from the reference sources where
  they lie and compiled with gcc.  The Cython step runs only where the reference
  tree and Cython exist; the generated ``.c`` files then travel with the repo
  snapshot, so a machine without Cython (but with Python and numpy headers)
  still compiles the reference kernels from them.  ``Extra_funs`` imports tqdm
  at module load, so it is built only where tqdm is importable.

The reference's own setup flags (``-mavx2 -m3dnow -march=native``) are x86
specific; this recipe uses ``-O3 -fopenmp`` so the result is the same code on
both architectures.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libkpm_oracle.so")
# The reference source tree (read-only); KPM_REFERENCE_ROOT points elsewhere if it lives there.
REFERENCE_ROOT = os.environ.get("KPM_REFERENCE_ROOT", "/root/reference")
REF_PYX = {
    "blas_funs": os.path.join(REFERENCE_ROOT, "jclsquant", "cython_modules", "blas_funs.pyx"),
    "Extra_funs": os.path.join(REFERENCE_ROOT, "jclsquant", "cython_modules", "Extra_funs.pyx"),
}


def _newer(src: str, dst: str) -> bool:
    return not os.path.exists(dst) or os.path.getmtime(src) > os.path.getmtime(dst)


def build_oracle(force: bool = False) -> str:
    """Compile kpm_oracle.c into oracle/_build/libkpm_oracle.so; return its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    src = os.path.join(HERE, "kpm_oracle.c")
    if force or _newer(src, ORACLE_SO):
        tmp = ORACLE_SO + ".tmp"
        cmd = ["gcc", "-O2", "-std=gnu99", "-fopenmp", "-fPIC", "-shared", src, "-o", tmp, "-lm"]
        subprocess.run(cmd, check=True)
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def _ext_suffix() -> str:
    return sysconfig.get_config_var("EXT_SUFFIX") or ".so"


def ref_module_path(name: str) -> str:
    return os.path.join(REF_DIR, name + _ext_suffix())


def _cythonize(name: str) -> str | None:
    """Translate a reference .pyx into oracle/_ref/<name>.c (only where the reference exists)."""
    pyx = REF_PYX[name]
    c_out = os.path.join(REF_DIR, name + ".c")
    if not os.path.exists(pyx):
        return c_out if os.path.exists(c_out) else None
    try:
        import Cython  # noqa: F401
    except ImportError:
        return c_out if os.path.exists(c_out) else None
    if _newer(pyx, c_out):
        os.makedirs(REF_DIR, exist_ok=True)
        subprocess.run([sys.executable, "-m", "cython", "-3", "--fast-fail", pyx, "-o", c_out],
                       check=True, stdout=subprocess.DEVNULL)
    return c_out


def build_reference(names=("blas_funs", "Extra_funs"), force: bool = False) -> dict:
    """Build the reference's Cython kernels into oracle/_ref; return {name: path or None}."""
    out = {}
    try:
        import numpy
        np_inc = numpy.get_include()
    except Exception:  # pragma: no cover - numpy is always present in practice
        return {n: None for n in names}
    py_inc = sysconfig.get_paths()["include"]
    if not os.path.exists(os.path.join(py_inc, "Python.h")):
        return {n: None for n in names}
    for name in names:
        if name == "Extra_funs":
            try:
                import tqdm  # noqa: F401
            except ImportError:
                out[name] = None
                continue
        c_src = _cythonize(name)
        if c_src is None or not os.path.exists(c_src):
            out[name] = None
            continue
        so = ref_module_path(name)
        if force or _newer(c_src, so):
            tmp = so + ".tmp"
            cmd = ["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-DNPY_NO_DEPRECATED_API=NPY_1_7_API_VERSION",
                   "-I" + py_inc, "-I" + np_inc, c_src, "-o", tmp, "-lm"]
            r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
            if r.returncode != 0:
                sys.stderr.write("reference kernel %s did not compile:\n%s\n" % (name, r.stdout[-2000:]))
                out[name] = None
                continue
            os.replace(tmp, so)
        out[name] = so
    return out


def clean() -> None:
    for d in (BUILD_DIR,):
        if os.path.isdir(d):
            shutil.rmtree(d)


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
