"""Build recipe of libsgfim.so and the CLI shims (nvcc, sm_103a, no cmake).

Every translation unit is compiled in parallel with
``-gencode arch=compute_103a,code=sm_103a``; the objects are linked into
``sgfim/_lib/libsgfim.so`` inside the source tree, next to the Python binding
that loads it.  Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")
OUT = os.path.join(PKG, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libsgfim.so")
CLI_SRC = {"sgfim_tensorfim": "cli_tensorfim.cpp", "sgfim_anytime": "cli_anytime.cpp"}

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags():
    return ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
            "-I", CSRC, "-I", INCLUDE] + ARCH


def _headers():
    return glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, extra):
    obj = os.path.join(OBJ, os.path.basename(src) + ".o")
    deps = [src] + _headers()
    if not _stale(obj, deps):
        return obj, None
    cmd = [nvcc(), "-c", src, "-o", obj] + _flags() + extra
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "c++", "-c", src, "-o", obj, "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
               "-I", CSRC, "-I", INCLUDE]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    return obj, p.stderr


def build(verbose=False, extra=None, jobs=None):
    """Compile every source under csrc/ and link libsgfim.so; returns its path."""
    os.makedirs(OBJ, exist_ok=True)
    extra = list(extra or [])
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    srcs = [s for s in srcs if not os.path.basename(s).startswith("cli_")]
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        res = list(ex.map(lambda s: _compile(s, extra), srcs))
    objs = [o for o, _ in res]
    if verbose:
        for _, log in res:
            if log:
                sys.stderr.write(log)
    if _stale(LIB, objs):
        cmd = [nvcc(), "-shared", "-o", LIB] + objs + ARCH + ["-lcudart", "-lpthread"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    for exe, src in CLI_SRC.items():
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        target = os.path.join(OUT, exe)
        if _stale(target, [s, LIB] + _headers()):
            cmd = [nvcc(), "-x", "c++", "-O2", "-std=c++17", s, "-o", target, "-I", INCLUDE,
                   "-L", OUT, "-lsgfim", "-Xlinker", "-rpath", "-Xlinker", "$ORIGIN"]
            p = subprocess.run(cmd, capture_output=True, text=True)
            if p.returncode != 0:
                raise RuntimeError(f"cli build failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    return LIB


def ptxas_report():
    """Registers / spills / shared memory per kernel (``-Xptxas -v``)."""
    out = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        cmd = [nvcc(), "-c", src, "-o", os.devnull] + _flags() + ["-Xptxas", "-v"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        out.append(p.stderr)
    return "\n".join(out)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "ptxas":
        print(ptxas_report())
    else:
        print(build(verbose=True))
