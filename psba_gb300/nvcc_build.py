"""Build recipe for the CUDA library (sm_103a).

Compiles ``csrc/*.cu`` with nvcc into ``psba_gb300/libpsba_gb300.so``: one
``-gencode`` (compute_103a / sm_103a), translation units compiled in
parallel, then linked with the static CUDA runtime.  No CMake.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpsba_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".h")]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return r.stdout + r.stderr


def build(force=False, verbose=False, extra=()):
    srcs = sources()
    newest = max(os.path.getmtime(f) for f in srcs + headers() + [__file__])
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    flags = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC] + ARCH
    flags += list(extra)
    objs = []

    def one(src):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        out = _run([nvcc()] + flags + ["-c", src, "-o", obj] +
                   (["-Xptxas", "-v"] if verbose else []))
        return obj, out

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(one, srcs))
    for obj, out in results:
        objs.append(obj)
        if verbose and out:
            sys.stderr.write(out)
    tmp = LIB + ".tmp"
    _run([nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-cudart", "static"])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
