"""Build recipe for the CPU oracle (test infrastructure only).

Two shared libraries are produced:

* ``oracle/_build/liboracle.so`` -- the C restatement in ``wstack_oracle.c``.
  It is compiled wherever the tests run (here and on the GPU host).
* ``oracle/_ref/libref.so`` -- the reference's own CPU path, compiled straight
  from the reference tree (``w-stacking.cu`` and ``phase_correction.cu`` as C,
  ``-DPHASE_ON``, exactly as the reference's Makefile copies them to ``.c``).
  It is built only when the reference tree is present; its sources are never
  copied into this repository.

A third artefact, ``oracle/_ref/refio``, is the reference's own reader,
v-slab sectoring, single-rank gridding loop and grid dump writer
(``init.c``, ``allvars.c``, ``gridding.c`` and ``w-stacking.cu`` as C,
compiled where they lie with ``-DUSE_MPI -DWRITE_DATA`` and the
single-process stand-in header ``refshim/mpi.h``) driven by
``refio_main.c``; it is also built only when the reference tree is present.

The two shared libraries use the same flags (``-O2 -ffp-contract=off``) so that a single-threaded
run of one is bit-identical to the other on x86-64 and aarch64.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "liboracle.so")
REF_SO = os.path.join(REF_DIR, "libref.so")
REFIO = os.path.join(REF_DIR, "refio")


def _reference_tree() -> str:
    """The reference checkout: ``--reference-tree DIR`` on the command line,
    else ``WSTACK_REFERENCE_TREE``, else a ``reference/`` checkout beside this
    repository.  Where none holds the sources, the reference builds are
    skipped and the tests that pin the oracle to them skip too."""
    for i, a in enumerate(sys.argv[:-1]):
        if a == "--reference-tree":
            return os.path.abspath(sys.argv[i + 1])
    env = os.environ.get("WSTACK_REFERENCE_TREE")
    if env:
        return os.path.abspath(env)
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


REFERENCE_TREE = _reference_tree()

CFLAGS = ["-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared"]


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources)


def build_oracle(force: bool = False) -> str:
    src = os.path.join(HERE, "wstack_oracle.c")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not _newer(ORACLE_SO, [src, __file__]):
        cmd = ["gcc", *CFLAGS, src, "-o", ORACLE_SO, "-lm"]
        subprocess.run(cmd, check=True)
    return ORACLE_SO


def reference_sources() -> list[str] | None:
    srcs = [os.path.join(REFERENCE_TREE, f) for f in ("w-stacking.cu", "phase_correction.cu")]
    if all(os.path.exists(s) for s in srcs):
        return srcs
    return None


def build_ref(force: bool = False) -> str | None:
    """Compile the reference's CPU gridding + phase correction, if present."""
    srcs = reference_sources()
    if srcs is None:
        return REF_SO if os.path.exists(REF_SO) else None
    os.makedirs(REF_DIR, exist_ok=True)
    if force or not _newer(REF_SO, srcs + [__file__]):
        # -x c: the reference's Makefile copies these .cu files to .c and
        # compiles them with the C compiler (Makefile:51-55); the __CUDACC__
        # branches are then excluded and the OpenMP CPU bodies are used.
        cmd = ["gcc", "-x", "c", *CFLAGS, "-DPHASE_ON", f"-I{REFERENCE_TREE}", *srcs,
               "-x", "none", "-o", REF_SO, "-lm"]
        subprocess.run(cmd, check=True)
    return REF_SO


def build_refio(force: bool = False) -> str | None:
    """Compile the reference's reader (init.c, allvars.c) with refio_main.c, if present.

    The reference compiles these files with -DUSE_MPI (Makefile:23); its
    non-MPI branch of init.c does not compile (allocate_memory names
    undeclared variables).  With one process every MPI call in them is a
    broadcast or a barrier, which refshim/mpi.h turns into no-ops."""
    srcs = [os.path.join(REFERENCE_TREE, f) for f in ("init.c", "allvars.c", "gridding.c")]
    wstack_src = os.path.join(REFERENCE_TREE, "w-stacking.cu")
    if not all(os.path.exists(s) for s in srcs + [wstack_src]):
        return REFIO if os.path.exists(REFIO) else None
    main_c = os.path.join(HERE, "refio_main.c")
    shim = os.path.join(HERE, "refshim", "mpi.h")
    os.makedirs(REF_DIR, exist_ok=True)
    if force or not _newer(REFIO, srcs + [wstack_src, main_c, shim, __file__]):
        # -ffp-contract=off as for libref.so: the gridding sums are then the
        # reference's exact operations on both host architectures
        cmd = ["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-DUSE_MPI", "-DWRITE_DATA", "-w",
               f"-I{os.path.join(HERE, 'refshim')}", f"-I{REFERENCE_TREE}", main_c, *srcs,
               "-x", "c", wstack_src, "-x", "none", "-o", REFIO, "-lm"]
        subprocess.run(cmd, check=True)
    return REFIO


def main() -> int:
    force = "--force" in sys.argv
    print(build_oracle(force))
    print(build_ref(force))
    print(build_refio(force))
    return 0


if __name__ == "__main__":
    sys.exit(main())
