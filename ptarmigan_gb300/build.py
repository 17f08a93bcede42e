"""Builds the engine's shared library, in-tree, for sm_103a only.

``build()`` runs nvcc on ``csrc/ptg_engine.cu`` (one translation unit that
includes every kernel) into ``_build/libptarmigan_gb300.so``.  It rebuilds
only when a source is newer than the library.
"""

import glob
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libptarmigan_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _sources():
    srcs = glob.glob(os.path.join(HERE, "csrc", "*.cu")) + glob.glob(os.path.join(HERE, "csrc", "*.cuh"))
    srcs += [os.path.join(HERE, "tables", "ptg_tables_small.h"), os.path.join(ROOT, "include", "ptarmigan_gb300.h")]
    return srcs


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine must be compiled with the CUDA toolkit")


def needs_build():
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    return any(os.path.getmtime(s) > t for s in _sources())


def build(force=False, verbose=False):
    """Compiles the library if needed and returns its path."""
    if not force and not needs_build():
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp"
    cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-shared",
           "-diag-suppress", "20091", "-o", tmp, os.path.join(HERE, "csrc", "ptg_engine.cu")]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + out.stdout + out.stderr)
    if verbose:
        print(out.stdout + out.stderr)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH
