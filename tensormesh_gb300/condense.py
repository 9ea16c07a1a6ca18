"""Dirichlet static condensation with the reference's interface
(operator/condense.py:26-443): ``Condenser(mask, value)``, ``__call__(K, b)``
-> (K_ii, b_i - K_io u_o), ``condense_rhs``, ``recover``, ``restrict``,
``prolong``, ``update_dirichlet``.

The edge masks and local numbering are computed once per sparsity layout and
cached; every call after that is one ``tm_condense`` launch (the K_ii and K_io
value gathers and rhs_i - K_io u_o together) on the cached index arrays, with
no host synchronisation and no host hashing.  The condensed matrices reuse
the cached index arrays and their CSR structure.
"""
import ctypes
from typing import Optional, Tuple

import numpy as np
import torch
import torch.nn as nn

from . import _lib
from .sparse import SparseMatrix


class _CondenseFn(torch.autograd.Function):
    """tm_condense with gradients: d/d values is a copy of the output
    gradients to their (distinct) source positions plus -u_o times the row
    gradient at the K_io positions; d/d rhs is the output gradient at the
    inner dofs; d/d u_o is -K_io^T times the row gradients."""

    @staticmethod
    def forward(ctx, cond, values, rhs, uo, row_src, with_mats):
        kept, io_vals, f_inner = cond._launch(values, rhs, with_mats, with_mats, row_src, uo)
        ctx.cond, ctx.row_src, ctx.with_mats = cond, row_src, with_mats
        ctx.shapes = (values.shape, rhs.shape)
        ctx.save_for_backward(values, uo)
        return kept, io_vals, f_inner

    @staticmethod
    def backward(ctx, g_kept, g_io, g_f):
        cond, row_src = ctx.cond, ctx.row_src
        values, uo = ctx.saved_tensors
        vshape, rshape = ctx.shapes
        n_inner = cond._k_inner_dof.numel()
        gf = g_f.reshape(n_inner, -1) if g_f is not None else None
        gsum = gf.sum(1) if gf is not None else None
        g_vals = g_rhs = g_uo = None
        if ctx.needs_input_grad[1]:
            g_vals = torch.zeros(vshape, dtype=values.dtype, device=values.device).reshape(-1)
            if ctx.with_mats and g_kept is not None:
                g_vals[cond._k_kept] = g_kept.reshape(-1)
            if ctx.with_mats and g_io is not None:
                g_vals[cond._k_io] = g_io.reshape(-1)
            if gsum is not None and row_src.numel():
                row_of = torch.repeat_interleave(torch.arange(n_inner, device=values.device),
                                                 cond._k_row_ptr[1:] - cond._k_row_ptr[:-1])
                g_vals[row_src] += -uo[cond._k_row_col] * gsum[row_of]
            g_vals = g_vals.reshape(vshape)
        if ctx.needs_input_grad[2] and gf is not None:
            g_rhs = torch.zeros(rshape[0], gf.shape[1], dtype=gf.dtype, device=gf.device)
            g_rhs[cond._k_inner_dof] = gf
            g_rhs = g_rhs.reshape(rshape)
        if ctx.needs_input_grad[3] and gsum is not None and row_src.numel():
            row_of = torch.repeat_interleave(torch.arange(n_inner, device=values.device),
                                             cond._k_row_ptr[1:] - cond._k_row_ptr[:-1])
            g_uo = torch.zeros_like(uo).index_add_(0, cond._k_row_col, -values.reshape(-1)[row_src] * gsum[row_of])
        return None, g_vals, g_rhs, g_uo, None, None


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
        # scalar entries of the K_io blocks: row (inner node, a), column (outer node, b)
        hh = torch.arange(H, device=dev)
        srow = (local[br[blk_out]][:, None, None] * H + hh[None, :, None]).expand(-1, H, H).reshape(-1)
        scol = (local[bc[blk_out]][:, None, None] * H + hh[None, None, :]).expand(-1, H, H).reshape(-1)
        self._kernel_layout(torch.nonzero(~mask).reshape(-1), srow, scol, ni_n * H)
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
        self._kernel_layout(torch.nonzero(inner).reshape(-1), self.ou2in_row, self.ou2in_col, ni)
        self.is_inner_dof, self.is_outer_dof = inner, mask
        self.inner_shape, self.ou2in_shape = (ni, ni), (ni, no)
        self.n_inner_dof, self.n_outer_dof, self.n_dof = ni, no, matrix.shape[0]
        self.layout_hash = matrix.layout_hash
        self._sorted = bool(matrix._sorted) and matrix._block == 1
        self._K_template = None
        self._Kio_template = None

    def _kernel_layout(self, inner_dof, io_row, io_col, n_inner):
        """Index arrays of tm_condense: the K_io entries (in K_io's own order,
        io_row / io_col their inner row and outer column) re-listed by inner
        row, stably, as positions in the full values (row_src) and in the
        K_io values (row_src_io)."""
        # one-time host work (a stable sort and a count of the K_io rows)
        dev = io_row.device
        row_np = io_row.detach().cpu().numpy().astype(np.int64)
        order_np = np.argsort(row_np, kind="stable")
        counts = np.bincount(row_np, minlength=n_inner) if row_np.size else np.zeros(n_inner, dtype=np.int64)
        row_ptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
        order = torch.from_numpy(order_np).to(dev)
        self._k_inner_dof = inner_dof.long().contiguous()
        self._k_row_ptr = torch.from_numpy(row_ptr).to(dev)
        self._k_row_src_io = order.long().contiguous()
        self._k_row_src = self.ou2in_idx[order].long().contiguous()
        self._k_row_col = io_col[order].long().contiguous()
        self._k_kept = self.inner_idx.long().contiguous()
        self._k_io = self.ou2in_idx.long().contiguous()

    def _condense(self, values, rhs, row_src, with_mats):
        uo = self.dirichlet_value
        if torch.is_grad_enabled() and (values.requires_grad or rhs.requires_grad or uo.requires_grad):
            return _CondenseFn.apply(self, values, rhs, uo, row_src, with_mats)
        return self._launch(values, rhs, with_mats, with_mats, row_src, uo)

    def _launch(self, values, rhs, kept, io, row_src, uo):
        """One tm_condense call; returns (K_ii values, K_io values, f_i)."""
        dev, dt = values.device, values.dtype
        _lib.require_cuda(values, "matrix values")
        n_inner = self._k_inner_dof.numel()
        rhs2 = rhs.reshape(rhs.shape[0], -1).contiguous()
        W = rhs2.shape[1]
        out_kept = torch.empty(self._k_kept.numel() if kept else 0, dtype=dt, device=dev)
        out_io = torch.empty(self._k_io.numel() if io else 0, dtype=dt, device=dev)
        out_rhs = torch.empty(n_inner, W, dtype=dt, device=dev)
        uo = uo.detach().contiguous()
        values = values.detach().contiguous()
        rhs2 = rhs2.detach()
        a = _lib.CondenseArgs()
        a.dtype, a.width, a.values = _lib.dtype_code(dt), max(1, W), _lib.ptr(values)
        a.n_kept, a.kept_src, a.out_kept = out_kept.numel(), _lib.ptr(self._k_kept), _lib.ptr(out_kept)
        a.n_io, a.io_src, a.out_io = out_io.numel(), _lib.ptr(self._k_io), _lib.ptr(out_io)
        a.n_inner = n_inner if W > 0 else 0
        a.inner_dof, a.row_ptr = _lib.ptr(self._k_inner_dof), _lib.ptr(self._k_row_ptr)
        a.n_row_entries, a.row_src = row_src.numel(), _lib.ptr(row_src)
        a.row_col, a.outer_value = _lib.ptr(self._k_row_col), _lib.ptr(uo)
        a.rhs, a.out_rhs = _lib.ptr(rhs2), _lib.ptr(out_rhs)
        _lib.check(_lib.load().tm_condense(ctypes.byref(a), _lib.stream_handle(dev)), "tm_condense")
        return out_kept, out_io, out_rhs.reshape(n_inner, *rhs.shape[1:])

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
        self.dirichlet_value = self.dirichlet_value.to(dtype=vals.dtype, device=vals.device)
        rhs = rhs.to(dtype=vals.dtype, device=vals.device)
        kept, io_vals, f_inner = self._condense(vals.reshape(-1), rhs, self._k_row_src, True)
        if self._K_template is None and self._blocks is not None:
            H, ir, ic, orow, ocol, ni_n, no_n = self._blocks
            self._K_template = SparseMatrix.from_block_coo(kept.view(-1, H, H), ir, ic, (ni_n, ni_n))
            self._K_template._sorted = self._sorted or None
            self._Kio_template = SparseMatrix.from_block_coo(io_vals.view(-1, H, H), orow, ocol, (ni_n, no_n))
            self._Kio_template._sorted = self._sorted or None
            K_inner, K_ou2in = self._K_template, self._Kio_template
        elif self._K_template is None:
            self._K_template = SparseMatrix(kept, self.inner_row, self.inner_col, self.inner_shape,
                                            _sorted=self._sorted or None)
            self._Kio_template = SparseMatrix(io_vals, self.ou2in_row, self.ou2in_col, self.ou2in_shape,
                                              _sorted=self._sorted or None)
            K_inner, K_ou2in = self._K_template, self._Kio_template
        else:
            H = self._blocks[0] if self._blocks is not None else 1
            K_inner = self._K_template.with_values(kept.view(-1, H, H) if H > 1 else kept)
            K_ou2in = self._Kio_template.with_values(io_vals.view(-1, H, H) if H > 1 else io_vals)
        self.K_ou2in = K_ou2in
        return K_inner, f_inner

    def condense_rhs(self, rhs: torch.Tensor) -> torch.Tensor:
        assert self.K_ou2in is not None, \
            "call the Condenser on a matrix first; condense_rhs reuses the cached K_io block"
        io_vals = self.K_ou2in.values
        rhs = rhs.to(dtype=io_vals.dtype, device=io_vals.device)
        self.dirichlet_value = self.dirichlet_value.to(dtype=rhs.dtype, device=rhs.device)
        _, _, f_inner = self._condense(io_vals.reshape(-1), rhs, self._k_row_src_io, False)
        return f_inner

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
