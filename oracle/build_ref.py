"""TEST INFRASTRUCTURE -- builds the reference UltimateKalman C library for the
golden fixtures.

Compiles the reference's own C sources where they lie (/root/reference/c) into
oracle/_ref/libukref.so, linked against the LAPACK/BLAS that SciPy bundles
(libscipy_openblas, whose exported symbols carry a ``scipy_`` prefix, hence the
-D renames).  The sequential parallel backend (c/parallel_sequential.c) is used.

One source line is patched, in a temporary copy outside the repository: in
c/kalman_oddeven_smoother.c the odd-length fix-up frees G_tilde (line 1469)
and then reads its dimensions (line 1471); the read is moved above the free.
Without it every odd-length recursion level aborts.

The result is x86-only and never travels as product: tests read the fixtures
it produced (tests/golden/*.npz), not the library.  Usage:
    python oracle/build_ref.py
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
import tempfile

# the reference C sources: UKG_REFERENCE_C, else where the build machine keeps them
REF_C = os.environ.get("UKG_REFERENCE_C", "/root/reference/c")
HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
OUT_LIB = os.path.join(OUT_DIR, "libukref.so")

SOURCES = [
    "kalman_ultimate.c", "kalman_conventional.c", "kalman_oddeven_smoother.c", "kalman_associative_smoother.c",
    "kalman_base.c", "kalman_explicit_representation.c", "matrix_ops.c", "flexible_arrays.c", "concurrent_set.c",
    "parallel_sequential.c",
]
HEADERS = ["kalman.h", "matrix_ops.h", "flexible_arrays.h", "parallel.h", "concurrent_set.h", "memory.h"]


def sources_present():
    """True where the reference sources exist (the build machine only)."""
    return os.path.isdir(REF_C)


def find_openblas():
    import scipy
    libs = glob.glob(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs", "libscipy_openblas*.so"))
    if not libs:
        raise FileNotFoundError("libscipy_openblas not found next to scipy")
    return os.path.abspath(libs[0])


def patch_oddeven(text: str) -> str:
    """Moves the read of G_tilde's dimensions above the free that precedes it."""
    free_line = "free_and_assign(&(step_lmo->G_tilde), R);"
    read_line = "int32_t ll = MAX(matrix_rows(G_tilde), matrix_cols(G_tilde));"
    lines = text.split("\n")
    i_free = [i for i, l in enumerate(lines) if free_line in l]
    i_read = [i for i, l in enumerate(lines) if read_line in l]
    if len(i_free) != 1 or len(i_read) != 1 or not (i_free[0] < i_read[0]):
        raise RuntimeError("reference odd-even source does not have the expected fix-up lines")
    r = lines.pop(i_read[0])
    lines.insert(i_free[0], r)
    return "\n".join(lines)


def build(force=False):
    if os.path.exists(OUT_LIB) and not force:
        return OUT_LIB
    if not os.path.isdir(REF_C):
        raise FileNotFoundError(REF_C)
    blas = find_openblas()
    os.makedirs(OUT_DIR, exist_ok=True)
    defs = ["-DBUILD_BLAS_UNDERSCORE", "-DBUILD_BLAS_STRLEN_END",
            "-DKALMAN_STEP_INDEX_TYPE_INT32", "-DFARRAY_INDEX_TYPE_INT32", "-DPARALLEL_INDEX_TYPE_INT32"]
    for f in ("dgemm_", "dgeqrf_", "dormqr_", "dtrtrs_", "dpotrf_"):
        defs.append(f"-D{f}=scipy_{f}")
    with tempfile.TemporaryDirectory(prefix="ukref_") as tmp:
        srcs = []
        for h in HEADERS:
            shutil.copy(os.path.join(REF_C, h), tmp)
        for s in SOURCES:
            text = open(os.path.join(REF_C, s)).read()
            if s == "kalman_oddeven_smoother.c":
                text = patch_oddeven(text)
            dst = os.path.join(tmp, s)
            open(dst, "w").write(text)
            srcs.append(dst)
        cmd = ["gcc", "-O2", "-fPIC", "-shared", "-w", "-o", OUT_LIB + ".tmp", *defs, *srcs,
               blas, f"-Wl,-rpath,{os.path.dirname(blas)}", "-lm"]
        subprocess.run(cmd, check=True)
    os.replace(OUT_LIB + ".tmp", OUT_LIB)
    return OUT_LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
