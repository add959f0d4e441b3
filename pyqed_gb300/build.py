"""Build the CUDA library ``pyqed_gb300/_lib/liblindblad_gb300.so`` for sm_103a.

Plain ``nvcc`` (no cmake, no torch extension machinery): every ``csrc/*.cu``
is compiled to an object in parallel, then linked into one shared library
with the CUDA runtime linked statically.  Rebuilds only when a source, a
header or the flags changed (a stamp file holds their hash).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
LIBDIR = os.path.join(HERE, "_lib")
OBJDIR = os.path.join(LIBDIR, "obj")
LIBNAME = "liblindblad_gb300.so"
LIBPATH = os.path.join(LIBDIR, LIBNAME)
CUDA_LIB = "/usr/local/cuda/lib64"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-O2",
              "--expt-relaxed-constexpr", "-I" + INCLUDE, "-I" + CSRC] + ARCH


def _nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pyqed_gb300")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stamp(files):
    h = hashlib.sha256()
    h.update(" ".join(NVCC_FLAGS).encode())
    deps = files + sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC)
                          if f.endswith((".cuh", ".h")))
    deps += [os.path.join(INCLUDE, f) for f in sorted(os.listdir(INCLUDE))]
    for f in deps:
        h.update(f.encode())
        with open(f, "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()


def build(verbose=False, force=False):
    """Compile and link the library; returns its path."""
    srcs = _sources()
    stamp = _stamp(srcs)
    stamp_file = os.path.join(LIBDIR, "stamp.txt")
    if (not force and os.path.exists(LIBPATH) and os.path.exists(stamp_file)
            and open(stamp_file).read() == stamp):
        return LIBPATH
    os.makedirs(OBJDIR, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(OBJDIR, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose:
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIBPATH + ".tmp"
    cmd = ([nvcc, "-shared"] + ARCH + ["-cudart", "static", "-o", tmp] + objs +
           ["-L" + CUDA_LIB, "-lcublas", "-Xlinker", "-rpath=" + CUDA_LIB])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIBPATH)
    with open(stamp_file, "w") as fh:
        fh.write(stamp)
    return LIBPATH


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
