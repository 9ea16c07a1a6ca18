"""The oracle's restatement of the reference's Jacobi-BiCGSTAB
(sparse/solve/torch_solve.py:130-248) against the reference's own solve of
a small non-symmetric system (tests/golden/small_krylov.npz, written by
make_golden.py --only=krylov), and the solver entry points exported by the
library (no GPU needed)."""
import os

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spl
import torch

from oracle import fem_oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "small_krylov.npz")


def _system():
    d = np.load(GOLDEN)
    n = d["b"].size
    A = sp.csr_matrix((d["values"], (d["row"], d["col"])), shape=(n, n))
    return d, A, n


def test_fixture_is_non_symmetric_and_solved():
    d, A, n = _system()
    assert abs(A - A.T).max() > 0.1
    xs = spl.spsolve(A.tocsc(), d["b"])
    assert np.linalg.norm(d["x"] - xs) <= 1e-12 * np.linalg.norm(xs)


def test_oracle_bicgstab_matches_reference():
    d, A, n = _system()
    t = lambda k: torch.from_numpy(d[k])
    x, it = O.reference_bicgstab(t("values"), t("row"), t("col"), n, t("b"), atol=1e-6, max_iter=2000)
    assert it < 2000
    assert np.linalg.norm(x.numpy() - d["x"]) <= 1e-11 * np.linalg.norm(d["x"])


def test_library_exports_bicgstab():
    from tensormesh_gb300 import _lib
    lib = _lib.load()
    for name in ("tm_bicgstab_start", "tm_bicgstab_iterate"):
        assert hasattr(lib, name)
