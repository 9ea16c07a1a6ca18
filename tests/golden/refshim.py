"""Minimal stand-ins for the two third-party packages the reference imports
at module load (``meshio`` and ``torch_sla``), so that the reference can be
imported on CPU to generate golden fixtures.

Only the attributes the reference's assembly path touches are provided:

* ``meshio.CellBlock`` / ``meshio.Mesh``: the container read by
  ``tensormesh/mesh/mesh.py:86-145`` (``cells``, ``cells_dict``,
  ``point_data``, ``cell_data``, ``cell_data_dict``, ``field_data``,
  ``cell_sets``).
* ``torch_sla.SparseTensor``: the COO base class of
  ``tensormesh/sparse/matrix.py:26`` (``values``, ``row_indices``,
  ``col_indices``, ``shape``, ``nnz``, ``to_dense``, ``@``) with a SciPy
  SuperLU ``solve``; torch-sla picks SuperLU on CPU as well
  (``docs/source/user_guide/batched_workflows.rst:127-129``).

This module is test infrastructure: it is used only by ``make_golden.py``.
"""
import sys
import types

import numpy as np


def install(reference_root: str) -> None:
    import torch
    import scipy.sparse
    import scipy.sparse.linalg

    if "meshio" not in sys.modules:
        meshio = types.ModuleType("meshio")

        class CellBlock:
            def __init__(self, type, data):
                self.type = type
                self.data = np.asarray(data)

        class Mesh:
            def __init__(self, points, cells, point_data=None, cell_data=None,
                         field_data=None, cell_sets=None):
                self.points = np.asarray(points)
                if isinstance(cells, dict):
                    cells = [CellBlock(k, v) for k, v in cells.items()]
                self.cells = [c if isinstance(c, CellBlock) else CellBlock(*c) for c in cells]
                self.point_data = dict(point_data or {})
                self.cell_data = dict(cell_data or {})
                self.field_data = dict(field_data or {})
                self.cell_sets = dict(cell_sets or {})

            @property
            def cells_dict(self):
                return {c.type: c.data for c in self.cells}

            @property
            def cell_data_dict(self):
                out = {}
                for key, blocks in self.cell_data.items():
                    out[key] = {c.type: v for c, v in zip(self.cells, blocks)}
                return out

        meshio.CellBlock = CellBlock
        meshio.Mesh = Mesh
        sys.modules["meshio"] = meshio

    if "torch_sla" not in sys.modules:
        sla = types.ModuleType("torch_sla")

        class SparseTensor:
            def __init__(self, values, row, col, shape):
                self.values = values
                self.row_indices = row
                self.col_indices = col
                self.shape = tuple(int(s) for s in shape)

            @property
            def nnz(self):
                return self.values.shape[0]

            @property
            def device(self):
                return self.values.device

            @property
            def dtype(self):
                return self.values.dtype

            def to_dense(self):
                out = torch.zeros(self.shape, dtype=self.values.dtype, device=self.values.device)
                out.index_put_((self.row_indices, self.col_indices), self.values, accumulate=True)
                return out

            def to_scipy(self):
                return scipy.sparse.coo_matrix(
                    (self.values.detach().cpu().numpy(),
                     (self.row_indices.cpu().numpy(), self.col_indices.cpu().numpy())),
                    shape=self.shape).tocsr()

            def __matmul__(self, x):
                out = torch.zeros(self.shape[0], *x.shape[1:], dtype=self.values.dtype, device=x.device)
                contrib = self.values.reshape(-1, *([1] * (x.dim() - 1))) * x[self.col_indices]
                return out.index_add(0, self.row_indices, contrib)

            def solve(self, b):
                A = self.to_scipy()
                x = scipy.sparse.linalg.spsolve(A.tocsc(), b.detach().cpu().numpy())
                return torch.from_numpy(np.asarray(x)).to(b.dtype)

        sla.SparseTensor = SparseTensor
        sys.modules["torch_sla"] = sla

    if reference_root not in sys.path:
        sys.path.insert(0, reference_root)
