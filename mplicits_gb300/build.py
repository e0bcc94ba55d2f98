"""Build libmplicits.so in-tree with nvcc for sm_103a.

``python -m mplicits_gb300.build`` (or ``build()``) compiles every ``.cu`` in
``csrc/`` in parallel into ``_build/`` and links ``libmplicits.so`` next to
this file.  Only stale objects are rebuilt.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
LIB = os.path.join(HERE, "libmplicits.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: libmplicits needs the CUDA toolkit to build")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return max(os.path.getmtime(h) for h in hs)


def _compile(src, verbose=False, extra=()):
    obj = os.path.join(BUILD, src[:-3] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-I", INCLUDE, "-I", CSRC, "-c",
           os.path.join(CSRC, src), "-o", obj + ".tmp"]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj, res.stderr


def build(force=False, verbose=False, jobs=None):
    """Compile stale translation units and relink; returns the library path."""
    os.makedirs(BUILD, exist_ok=True)
    hdr = _headers_mtime()
    todo = []
    objs = []
    for src in _sources():
        obj = os.path.join(BUILD, src[:-3] + ".o")
        objs.append(obj)
        if force or verbose or not os.path.exists(obj) or \
                os.path.getmtime(obj) < max(os.path.getmtime(os.path.join(CSRC, src)), hdr):
            todo.append(src)
    logs = []
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(8, len(todo))) as ex:
            for obj, log in ex.map(lambda s: _compile(s, verbose), todo):
                logs.append((obj, log))
    if todo or not os.path.exists(LIB):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcuda"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        for obj, log in logs:
            print(f"== {os.path.basename(obj)}\n{log}")
    return LIB


if __name__ == "__main__":
    path = build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(path)
