"""Build recipe for the oracle (test infrastructure only).

* ``build_oracle()`` compiles the C restatement ``psba_oracle.c`` into
  ``oracle/libpsba_oracle.so`` (gcc, -O2, no FMA contraction, OpenMP).
* ``build_ref()`` compiles the reference's own CPU-runnable sources where
  they lie (``PSBA/levmar_func_cpu.cpp`` and the barrier-free
  ``CL_files/*.cl`` kernels, pulled in by ``ref_shim.cpp``) into
  ``oracle/_ref/libpsba_ref.so``.  It only runs where the reference checkout
  exists; the output is git-ignored and is used to pin the oracle and to
  regenerate ``tests/golden``.
* ``build_ref_reader()`` compiles the reference's problem-file reader
  (``PSBA/readparams.cpp`` with ``quat2vec`` from ``PSBA/misc.cpp``, through
  ``ref_reader_shim.cpp``) into ``oracle/_ref/libpsba_ref_reader.so``, to pin
  this repository's reader against it.

The reference checkout is taken from ``PSBA_REFERENCE_DIR`` when it is set,
else from the path where this machine mounts it.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REFERENCE = os.environ.get("PSBA_REFERENCE_DIR", "/root/reference")
ORACLE_SO = os.path.join(HERE, "libpsba_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libpsba_ref.so")
REF_READER_SO = os.path.join(HERE, "_ref", "libpsba_ref_reader.so")


def reference_dir():
    """The reference checkout this recipe reads, or None where it is absent."""
    return REFERENCE if os.path.isdir(REFERENCE) else None


def reference_data_dir():
    """The reference's example problem files (data/), or None."""
    d = os.path.join(REFERENCE, "data")
    return d if os.path.isdir(d) else None


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("command failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle(force=False):
    src = os.path.join(HERE, "psba_oracle.c")
    hdr = os.path.join(HERE, "psba_oracle.h")
    if force or _stale(ORACLE_SO, [src, hdr, __file__]):
        _run(["gcc", "-O2", "-std=c99", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
              "-fPIC", "-shared", "-Wall", "-Wno-unused-variable", src, "-o", ORACLE_SO, "-lm"])
    return ORACLE_SO


def reference_available():
    return os.path.isfile(os.path.join(REFERENCE, "PSBA", "levmar_func_cpu.cpp")) and \
        os.path.isdir(os.path.join(REFERENCE, "CL_files"))


def build_ref(force=False):
    if not reference_available():
        return None
    os.makedirs(os.path.dirname(REF_SO), exist_ok=True)
    shim = os.path.join(HERE, "ref_shim.cpp")
    cpu = os.path.join(REFERENCE, "PSBA", "levmar_func_cpu.cpp")
    if force or _stale(REF_SO, [shim, __file__]):
        _run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
              "-shared", "-w", "-fpermissive",
              "-I" + os.path.join(REFERENCE, "CL_files"), "-I" + os.path.join(HERE, "ref_stub"),
              shim, cpu, "-o", REF_SO])
    return REF_SO


def build_ref_reader(force=False):
    src = os.path.join(REFERENCE, "PSBA", "readparams.cpp")
    if not (os.path.isfile(src) and os.path.isfile(os.path.join(REFERENCE, "PSBA", "misc.cpp"))):
        return None
    os.makedirs(os.path.dirname(REF_READER_SO), exist_ok=True)
    shim = os.path.join(HERE, "ref_reader_shim.cpp")
    if force or _stale(REF_READER_SO, [shim, __file__]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-w", "-fpermissive",
              "-I" + os.path.join(REFERENCE, "PSBA"), "-I" + os.path.join(HERE, "ref_stub"),
              shim, "-o", REF_READER_SO])
    return REF_READER_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_ref(force="--force" in sys.argv))
    print(build_ref_reader(force="--force" in sys.argv))
