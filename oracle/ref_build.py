"""Recipe: compile the reference's own factorization path into ``oracle/_ref/oocdag_ref``.

TEST INFRASTRUCTURE ONLY.  The reference project's ``oocdag.cpp`` (driver ``Cholesky``,
``find_Yn``, and ``main``, which is compiled under another name and never run) and
``oocquark.cpp`` (the task generators ``A2Y``/``A2X``/``ooc_syrk``/``ooc_incore`` and the
task bodies) are compiled unmodified, from where they lie in the reference tree, with the
reference's own build flags ``-DUSE_CUBLASV2 -DUSE_HOST_DPOTRF`` (its ``Makefile:6-8``).
Its third-party dependencies (QUARK, cuBLAS v2, the CUDA runtime, MPI_Wtime, MKL
``dpotrf_``, BLACS) are absent, so ``ref_shim/include`` stands in for their headers and
``ref_shim/shim.cpp`` implements them on the host (tasks in program order; BLAS/LAPACK
from SciPy's bundled OpenBLAS, loaded at run time).  Nothing is copied out of the
reference: only the compiled binary (``oracle/_ref``, git-ignored) is produced.

Runs only where the reference tree exists (``OOC_REFERENCE_DIR``, default the path
below); elsewhere ``build_ref`` returns None and the tests that need it skip.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
BIN = os.path.join(OUT_DIR, "oocdag_ref")
SHIM = os.path.join(HERE, "ref_shim")
DEFAULT_REFERENCE = "/root/reference"


def reference_dir() -> str:
    return os.environ.get("OOC_REFERENCE_DIR", DEFAULT_REFERENCE)


def available() -> bool:
    d = reference_dir()
    return all(os.path.exists(os.path.join(d, f)) for f in ("oocdag.cpp", "oocquark.cpp", "oocdag.h"))


def _inputs(ref: str) -> list[str]:
    shim = [os.path.join(SHIM, f) for f in ("shim.cpp", "shim.h", "ref_main.cpp")]
    shim += [os.path.join(SHIM, "include", f) for f in sorted(os.listdir(os.path.join(SHIM, "include")))]
    return shim + [os.path.join(ref, f) for f in ("oocdag.cpp", "oocquark.cpp", "oocdag.h")] + [__file__]


def build_ref(force: bool = False) -> str | None:
    """Compile the reference path; returns the binary's path, or None without the tree."""
    if not available():
        return None
    ref = reference_dir()
    if (not force and os.path.exists(BIN)
            and all(os.path.getmtime(p) <= os.path.getmtime(BIN) for p in _inputs(ref))):
        return BIN
    os.makedirs(OUT_DIR, exist_ok=True)
    cxx = shutil.which("g++") or "g++"
    common = [cxx, "-O2", "-std=c++17", "-w", "-DUSE_CUBLASV2", "-DUSE_HOST_DPOTRF",
              "-I" + os.path.join(SHIM, "include"), "-I" + SHIM, "-I" + ref]
    objs = []
    for src, extra in ((os.path.join(ref, "oocdag.cpp"), ["-Dmain=oocdag_reference_main"]),
                       (os.path.join(ref, "oocquark.cpp"), []),
                       (os.path.join(SHIM, "shim.cpp"), []),
                       (os.path.join(SHIM, "ref_main.cpp"), [])):
        obj = os.path.join(OUT_DIR, os.path.basename(src)[:-4] + ".o")
        subprocess.run(common + extra + ["-c", src, "-o", obj], check=True)
        objs.append(obj)
    subprocess.run([cxx, "-o", BIN + ".tmp", *objs, "-ldl"], check=True)
    os.replace(BIN + ".tmp", BIN)
    return BIN


if __name__ == "__main__":
    print(build_ref(force=True) or "reference tree not found: nothing built")
