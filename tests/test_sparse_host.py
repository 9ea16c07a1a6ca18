"""Host-side logic of SparseMatrix and of mixed-mesh element data (no GPU):
the transpose's CSR view built once per layout and shared by matrices of
that layout, the transpose's structure against a dense transpose, and the
split of element data over element types."""
import numpy as np
import torch

from tensormesh_gb300.assemble import _split_element_data
from tensormesh_gb300.sparse import SparseMatrix


def _random_matrix(n=7, nnz=20, seed=0):
    rng = np.random.default_rng(seed)
    keys = np.unique(rng.integers(0, n * n, nnz))
    row, col = torch.from_numpy(keys // n), torch.from_numpy(keys % n)
    vals = torch.from_numpy(rng.uniform(-1.0, 1.0, keys.size))
    return SparseMatrix(vals, row, col, (n, n), _sorted=True)


def test_transpose_structure_cached_per_layout():
    A = _random_matrix()
    T1 = A.transpose()
    T2 = A.transpose()
    assert T1._csr is T2._csr                       # built once
    B = A.with_values(A.values * 2.0)
    T3 = B.transpose()
    assert T3._csr is T1._csr                       # shared by the layout
    # the structure is that of the dense transpose
    rp, col, perm, H = T1._csr
    vals = T1.values if perm is None else T1.values[perm]
    dense = torch.zeros(A.shape, dtype=torch.float64)
    rows = torch.repeat_interleave(torch.arange(A.shape[0]), rp[1:] - rp[:-1])
    dense.index_put_((rows, col.long()), vals, accumulate=True)
    assert torch.equal(dense, A.to_dense().T)


def test_block_transpose_values():
    rng = np.random.default_rng(1)
    br = torch.tensor([0, 0, 1, 2])
    bc = torch.tensor([0, 2, 1, 0])
    v = torch.from_numpy(rng.uniform(-1.0, 1.0, (4, 2, 2)))
    A = SparseMatrix.from_block_coo(v, br, bc, (3, 3))
    assert torch.equal(A.transpose().to_dense(), A.to_dense().T)


class _Topo:
    types = ["quad", "triangle"]
    n_elements = {"quad": 3, "triangle": 2}


def test_split_element_data():
    flat = torch.arange(5.0)
    per = _split_element_data(_Topo(), {"kappa": flat, "E": {"quad": torch.ones(3), "triangle": torch.zeros(2)},
                                        "c": 2.5})
    assert torch.equal(per["quad"]["kappa"], flat[:3]) and torch.equal(per["triangle"]["kappa"], flat[3:])
    assert torch.equal(per["quad"]["E"], torch.ones(3)) and torch.equal(per["triangle"]["E"], torch.zeros(2))
    assert per["quad"]["c"] == 2.5 and per["triangle"]["c"] == 2.5
    # slicing keeps the autograd graph of a coefficient that requires grad
    k = torch.arange(5.0, requires_grad=True)
    per = _split_element_data(_Topo(), {"kappa": k})
    (per["quad"]["kappa"].sum() + 2.0 * per["triangle"]["kappa"].sum()).backward()
    assert torch.equal(k.grad, torch.tensor([1.0, 1.0, 1.0, 2.0, 2.0]))
