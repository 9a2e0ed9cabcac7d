"""Generate ``ref_run.npz``: factors computed by the compiled reference itself.

The reference's ``oocdag.cpp`` and ``oocquark.cpp`` are compiled unmodified by
``oracle/ref_build.py`` into ``oracle/_ref/oocdag_ref`` (host stand-ins for QUARK, cuBLAS
and MKL; see that file).  This script runs the reference's ``Cholesky`` on small seeded
matrices whose device budgets force several left-looking panels and ragged last tiles,
and stores each input's seed and sizes with the lower triangle of the factor (row-major
packed), so that the GPU tests can compare the library's factor with the reference's
own output on a machine where the reference tree is absent.

Run (where the reference tree exists):  python tests/golden/gen_ref_run.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import ref_build  # noqa: E402

# (name, n, nb, budget in tiles, generator)
CASES = [
    ("pdmatgen_n96_nb32_t7", 96, 32, 7, "pdmatgen"),
    ("uniform_n300_nb64_t14", 300, 64, 14, "uniform"),
    ("uniform_n200_nb48_t12", 200, 48, 12, "uniform"),
]


def matrix(n: int, kind: str) -> np.ndarray:
    return oracle.gen_pdmatgen(n, 100) if kind == "pdmatgen" else oracle.gen_uniform(n, 100, float(n))


def main() -> None:
    binary = ref_build.build_ref()
    if binary is None:
        raise SystemExit("the reference tree is needed to generate ref_run.npz")
    out = {}
    for name, n, nb, tiles, kind in CASES:
        A = matrix(n, kind)
        with tempfile.TemporaryDirectory() as d:
            fin, fout = os.path.join(d, "a.f64"), os.path.join(d, "l.f64")
            A.T.tofile(fin)
            r = subprocess.run([binary, "run", str(n), str(nb), str(n), str(tiles * nb * nb * 8),
                                oracle.openblas_path(), "scipy_", fin, fout], capture_output=True, text=True,
                               check=True)
            L = np.fromfile(fout, dtype=np.float64).reshape(n, n).T
        npanels = sum(1 for line in r.stdout.splitlines() if line.startswith("bb "))
        out[name] = L[np.tril_indices(n)]  # row-major packed lower triangle
        out[name + "_meta"] = np.array([n, nb, tiles, 0 if kind == "uniform" else 1, 100, npanels], dtype=np.int64)
    np.savez_compressed(os.path.join(HERE, "ref_run.npz"), **out)
    print("wrote", os.path.join(HERE, "ref_run.npz"), sorted(k for k in out if not k.endswith("_meta")))


if __name__ == "__main__":
    main()
