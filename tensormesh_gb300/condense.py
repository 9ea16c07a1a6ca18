"""Dirichlet static condensation with the reference's interface
(operator/condense.py:26-443): ``Condenser(mask, value)``, ``__call__(K, b)``
-> (K_ii, b_i - K_io u_o), ``condense_rhs``, ``recover``, ``restrict``,
``prolong``, ``update_dirichlet``.

The edge masks and local numbering are computed once per sparsity layout and
cached; the condensed matrices reuse the cached index arrays and their CSR
structure, so a repeated call does no host work and no host hashing.
"""
from typing import Optional, Tuple

import torch
import torch.nn as nn

from .sparse import SparseMatrix


class Condenser(nn.Module):
    def __init__(self, dirichlet_mask: torch.Tensor, dirichlet_value: Optional[torch.Tensor] = None):
        super().__init__()
        assert dirichlet_mask.dtype == torch.bool, f"dirichlet_mask must be a bool tensor, got {dirichlet_mask.dtype}"
        assert dirichlet_mask.ndim == 1, f"dirichlet_mask must be 1D, got shape {tuple(dirichlet_mask.shape)}"
        self.register_buffer("dirichlet_mask", dirichlet_mask)
        self.register_buffer("dirichlet_value", self._normalize_value(dirichlet_value))
        self.inner_row = None
        self._blocks = None
        self.layout_hash = None
        self.K_ou2in = None
        self.n_dof = None
        self.n_inner_dof = None
        self.n_outer_dof = None

    def _normalize_value(self, value):
        mask = self.dirichlet_mask
        n_outer = int(mask.sum())
        if value is None:
            return torch.zeros(n_outer, device=mask.device, dtype=torch.float64)
        assert value.ndim == 1, f"dirichlet_value must be 1D, got shape {tuple(value.shape)}"
        if value.shape[0] == mask.shape[0]:
            return value[mask]
        assert value.shape[0] == n_outer, \
            f"dirichlet_value must have length n_dof ({mask.shape[0]}) or n_outer_dof ({n_outer}), got {value.shape[0]}"
        return value

    def _compute_block_layout(self, matrix: SparseMatrix) -> bool:
        """Node-aligned masks on block matrices: condense whole HxH blocks.

        The kept scalar entries are exactly the entries of the kept blocks,
        in the same [block, a, b] order, so the values, rows and columns equal
        those of the scalar condensation while the result stays a block
        matrix (block-CSR SpMV, no index expansion)."""
        H = matrix._block
        dev = matrix.device
        mask = self.dirichlet_mask.to(dev)
        if H == 1 or mask.numel() % H:
            return False
        node_mask = mask.view(-1, H)
        if not bool((node_mask == node_mask[:, :1]).all()):
            return False
        nmask = node_mask[:, 0]
        br = matrix._block_row.to(dev).long()
        bc = matrix._block_col.to(dev).long()
        inner_n = ~nmask
        ib = inner_n[br] & inner_n[bc]
        ob = inner_n[br] & nmask[bc]
        ni_n, no_n = int(inner_n.sum()), int(nmask.sum())
        local = torch.full((nmask.numel(),), -1, dtype=torch.long, device=dev)
        local[inner_n] = torch.arange(ni_n, device=dev)
        local[nmask] = torch.arange(no_n, device=dev)
        blk_in = torch.nonzero(ib).reshape(-1)
        blk_out = torch.nonzero(ob).reshape(-1)
        k = torch.arange(H * H, device=dev)
        self.inner_idx = (blk_in[:, None] * (H * H) + k).reshape(-1)
        self.ou2in_idx = (blk_out[:, None] * (H * H) + k).reshape(-1)
        self._blocks = (H, local[br[blk_in]], local[bc[blk_in]], local[br[blk_out]], local[bc[blk_out]], ni_n, no_n)
        self.inner_row = None
        self.is_inner_dof, self.is_outer_dof = ~mask, mask
        self.inner_shape, self.ou2in_shape = (ni_n * H, ni_n * H), (ni_n * H, no_n * H)
        self.n_inner_dof, self.n_outer_dof, self.n_dof = ni_n * H, no_n * H, matrix.shape[0]
        self.layout_hash = matrix.layout_hash
        self._sorted = bool(matrix._sorted)
        self._K_template = None
        self._Kio_template = None
        return True

    def _compute_layout(self, matrix: SparseMatrix):
        self._blocks = None
        if self._compute_block_layout(matrix):
            return
        dev = matrix.device
        mask = self.dirichlet_mask.to(dev)
        edge_u, edge_v = matrix.row_indices, matrix.col_indices
        inner = ~mask
        iu, iv = inner[edge_u], inner[edge_v]
        is_inner_edge = iu & iv
        is_ou2in_edge = iu & mask[edge_v]
        ni, no = int(inner.sum()), int(mask.sum())
        local = torch.full((matrix.shape[0],), -1, dtype=torch.long, device=dev)
        local[inner] = torch.arange(ni, device=dev)
        local[mask] = torch.arange(no, device=dev)
        self.inner_idx = torch.nonzero(is_inner_edge).reshape(-1)
        self.ou2in_idx = torch.nonzero(is_ou2in_edge).reshape(-1)
        self.inner_row = local[edge_u[self.inner_idx]]
        self.inner_col = local[edge_v[self.inner_idx]]
        self.ou2in_row = local[edge_u[self.ou2in_idx]]
        self.ou2in_col = local[edge_v[self.ou2in_idx]]
        self.is_inner_dof, self.is_outer_dof = inner, mask
        self.inner_shape, self.ou2in_shape = (ni, ni), (ni, no)
        self.n_inner_dof, self.n_outer_dof, self.n_dof = ni, no, matrix.shape[0]
        self.layout_hash = matrix.layout_hash
        self._sorted = bool(matrix._sorted) and matrix._block == 1
        self._K_template = None
        self._Kio_template = None

    def update_dirichlet(self, dirichlet_value: torch.Tensor):
        self.dirichlet_value = self._normalize_value(dirichlet_value)

    def __call__(self, matrix: SparseMatrix, rhs: Optional[torch.Tensor] = None) -> Tuple[SparseMatrix, torch.Tensor]:
        if rhs is None:
            rhs = torch.zeros(matrix.shape[0], dtype=matrix.dtype, device=matrix.device)
        if self.n_dof is None:
            self._compute_layout(matrix)
        assert matrix.shape[0] == self.n_dof and matrix.shape[1] == self.n_dof, \
            f"the shape of matrix must be [{self.n_dof}, {self.n_dof}], but got {matrix.shape}"
        assert matrix.has_same_layout(self.layout_hash), \
            "the layout of the matrix is changed, please recompute the condensed matrix"
        assert rhs.shape[0] == self.n_dof, f"the shape of rhs must be [{self.n_dof}, ...], but got {rhs.shape}"
        vals = matrix.values
        if self._K_template is None and self._blocks is not None:
            H, ir, ic, orow, ocol, ni_n, no_n = self._blocks
            self._K_template = SparseMatrix.from_block_coo(vals[self.inner_idx].view(-1, H, H), ir, ic, (ni_n, ni_n))
            self._K_template._sorted = self._sorted or None
            self._Kio_template = SparseMatrix.from_block_coo(vals[self.ou2in_idx].view(-1, H, H), orow, ocol,
                                                             (ni_n, no_n))
            self._Kio_template._sorted = self._sorted or None
            K_inner, K_ou2in = self._K_template, self._Kio_template
        elif self._K_template is None:
            self._K_template = SparseMatrix(vals[self.inner_idx], self.inner_row, self.inner_col, self.inner_shape,
                                            _sorted=self._sorted or None)
            self._Kio_template = SparseMatrix(vals[self.ou2in_idx], self.ou2in_row, self.ou2in_col, self.ou2in_shape,
                                              _sorted=self._sorted or None)
            K_inner, K_ou2in = self._K_template, self._Kio_template
        else:
            K_inner = self._K_template.with_values(vals[self.inner_idx])
            K_ou2in = self._Kio_template.with_values(vals[self.ou2in_idx])
        self.K_ou2in = K_ou2in
        self.dirichlet_value = self.dirichlet_value.to(dtype=vals.dtype, device=vals.device)
        rhs = rhs.to(dtype=vals.dtype, device=vals.device)
        return K_inner, self._minus(rhs)

    def _minus(self, rhs):
        out = rhs[self.is_inner_dof]
        if self.n_outer_dof and bool((self.dirichlet_value != 0).any()):
            t = self.K_ou2in @ self.dirichlet_value
            for _ in range(rhs.dim() - 1):
                t = t.unsqueeze(-1)
            out = out - t
        return out

    def condense_rhs(self, rhs: torch.Tensor) -> torch.Tensor:
        assert self.K_ou2in is not None, \
            "call the Condenser on a matrix first; condense_rhs reuses the cached K_io block"
        rhs = rhs.to(dtype=self.K_ou2in.dtype, device=self.K_ou2in.device)
        self.dirichlet_value = self.dirichlet_value.to(dtype=rhs.dtype, device=rhs.device)
        return self._minus(rhs)

    def recover(self, u: torch.Tensor) -> torch.Tensor:
        assert u.shape[0] == self.n_inner_dof, f"the shape of u must be [{self.n_inner_dof}, ...], but got {u.shape}"
        shape = list(u.shape)
        shape[0] = self.n_dof
        u_full = torch.zeros(shape, dtype=u.dtype, device=u.device)
        u_full[self.is_inner_dof.to(u.device)] = u
        bv = self.dirichlet_value.to(dtype=u.dtype, device=u.device)
        for _ in range(u.dim() - 1):
            bv = bv.unsqueeze(-1)
        u_full[self.is_outer_dof.to(u.device)] += bv
        return u_full

    def restrict(self, f: torch.Tensor) -> torch.Tensor:
        assert f.shape[0] == self.dirichlet_mask.shape[0]
        return f[~self.dirichlet_mask.to(f.device)]

    def prolong(self, f_inner: torch.Tensor) -> torch.Tensor:
        mask = self.dirichlet_mask.to(f_inner.device)
        n_inner = int((~mask).sum())
        assert f_inner.shape[0] == n_inner
        shape = list(f_inner.shape)
        shape[0] = mask.shape[0]
        out = torch.zeros(shape, dtype=f_inner.dtype, device=f_inner.device)
        out[~mask] = f_inner
        return out
