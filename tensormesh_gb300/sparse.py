"""``SparseMatrix``: the COO container the assemblers return.

Mirrors ``tensormesh.sparse.SparseMatrix`` (sparse/matrix.py:26-381): the
constructor ``SparseMatrix(edata, row, col, shape)``, the attributes
``values``/``edata``, ``row_indices``/``row`` (int64), ``col_indices``/``col``,
``shape``, ``nnz``, ``edges``, ``layout_hash`` and ``has_same_layout``,
``to_dense``, ``@`` and ``solve``, and ``from_block_coo``.

Differences that do not change results:

* The reference hashes the (row, col) bytes on the host on every
  construction (sparse/matrix.py:82-86).  Here the SHA-256 of the same bytes
  is computed on first access and, for matrices produced by an assembler,
  once per mesh.
* Block matrices (``from_block_coo``) keep their [n_block, H, H] values and
  expand the scalar row/col indices only when asked.
* ``@`` runs the library's CSR / block-CSR SpMV kernels; ``solve`` runs the
  Jacobi-preconditioned CG of ``tensormesh_gb300.solve`` (the reference
  delegates to torch-sla, which picks a direct or iterative backend).
"""
import hashlib
from typing import Optional, Tuple

import numpy as np
import torch

from . import _lib


def block_layout_hash(block_row: torch.Tensor, block_col: torch.Tensor, H: int, slice_blocks: int = 1 << 20) -> str:
    """SHA-256 of the int64 scalar rows (block_row * H + a), then the scalar
    columns (block_col * H + b), in [block, a, b] order -- the bytes of the
    expanded matrix's row and column arrays -- hashed slice by slice."""
    h = hashlib.sha256()
    a = torch.arange(H, dtype=torch.long).repeat_interleave(H)
    b = torch.arange(H, dtype=torch.long).repeat(H)
    for src, off in ((block_row, a), (block_col, b)):
        src = src.detach()
        off = off.to(src.device)
        for s0 in range(0, src.numel(), slice_blocks):
            part = (src[s0:s0 + slice_blocks].long()[:, None] * H + off).reshape(-1)
            h.update(part.cpu().numpy().tobytes())
    return h.hexdigest()


class SparseMatrix:
    def __init__(self, edata: torch.Tensor, row: torch.Tensor, col: torch.Tensor,
                 shape: Tuple[int, int], *, _topology=None, _block: int = 1,
                 _block_row: Optional[torch.Tensor] = None, _block_col: Optional[torch.Tensor] = None,
                 _sorted: Optional[bool] = None):
        self.values = edata
        self._row_src = row
        self._col_src = col
        self.shape = (int(shape[0]), int(shape[1]))
        self._topology = _topology
        self._block = int(_block)
        self._block_row = _block_row
        self._block_col = _block_col
        self._row64 = None
        self._col64 = None
        self._hash = None
        self._sorted = _sorted
        self._csr = None
        self._order = None
        self._tstruct = {}     # the transpose's CSR view, shared by matrices of this layout

    # ------------------------------------------------------------ attributes
    @property
    def edata(self) -> torch.Tensor:
        return self.values

    @property
    def row_indices(self) -> torch.Tensor:
        if self._row64 is None:
            if self._block > 1:
                self._row64, self._col64 = self._expand_block()
            else:
                self._row64 = self._row_src.long()
        return self._row64

    @property
    def col_indices(self) -> torch.Tensor:
        if self._col64 is None:
            if self._block > 1:
                self._row64, self._col64 = self._expand_block()
            else:
                self._col64 = self._col_src.long()
        return self._col64

    row = row_indices
    col = col_indices

    @property
    def edges(self) -> torch.Tensor:
        return torch.stack([self.row_indices, self.col_indices], 0)

    @property
    def nnz(self) -> int:
        return int(self.values.numel())

    @property
    def device(self) -> torch.device:
        return self.values.device

    @property
    def dtype(self) -> torch.dtype:
        return self.values.dtype

    @property
    def layout_hash(self) -> str:
        """SHA-256 of the row bytes followed by the column bytes as passed to
        the constructor (sparse/matrix.py:82-86); for block matrices, of the
        expanded int64 scalar rows and columns, computed in slices without
        materialising them and kept per block size on the mesh topology."""
        if self._hash is None:
            if self._topology is not None and self._block == 1:
                self._hash = self._topology.layout_hash
            elif self._block > 1 and self._topology is not None:
                self._hash = self._topology.block_layout_hash(self._block)
            elif self._block > 1:
                self._hash = block_layout_hash(self._block_row, self._block_col, self._block)
            else:
                self._hash = hashlib.sha256(self._row_src.detach().cpu().numpy().tobytes()
                                            + self._col_src.detach().cpu().numpy().tobytes()).hexdigest()
        return self._hash

    def has_same_layout(self, other) -> bool:
        h = other if isinstance(other, str) else other.layout_hash
        return self.layout_hash == h

    # ---------------------------------------------------------- conversions
    def _expand_block(self):
        """row*H + a, col*H + b in [block, a, b] order (sparse/matrix.py:370-376)."""
        H = self._block
        br = self._block_row.to(self.values.device).long()
        bc = self._block_col.to(self.values.device).long()
        a = torch.arange(H, device=br.device).repeat_interleave(H)
        b = torch.arange(H, device=br.device).repeat(H)
        return ((br[:, None] * H + a).reshape(-1), (bc[:, None] * H + b).reshape(-1))

    @staticmethod
    def from_block_coo(edata: torch.Tensor, row: torch.Tensor, col: torch.Tensor,
                       shape: Tuple[int, int], *, _topology=None) -> "SparseMatrix":
        """Expand [n_block, H, H] block storage into an (N*H, N*H) matrix whose
        scalar entries are ordered [block, a, b] (sparse/matrix.py:332-381)."""
        H = int(edata.shape[1])
        assert edata.shape[2] == H, f"from_block_coo expects square blocks, got {tuple(edata.shape)}"
        return SparseMatrix(edata.reshape(-1), row, col, (shape[0] * H, shape[1] * H),
                            _topology=_topology, _block=H, _block_row=row, _block_col=col)

    def to_dense(self) -> torch.Tensor:
        out = torch.zeros(self.shape, dtype=self.values.dtype, device=self.values.device)
        out.index_put_((self.row_indices, self.col_indices), self.values, accumulate=True)
        return out

    def to_scipy_coo(self):
        import scipy.sparse
        return scipy.sparse.coo_matrix(
            (self.values.detach().cpu().numpy(),
             (self.row_indices.cpu().numpy(), self.col_indices.cpu().numpy())), shape=self.shape)

    def with_values(self, values: torch.Tensor) -> "SparseMatrix":
        """Same layout, new values (no re-hash, shared CSR structures)."""
        m = SparseMatrix(values, self._row_src, self._col_src, self.shape, _topology=self._topology,
                         _block=self._block, _block_row=self._block_row, _block_col=self._block_col,
                         _sorted=self._sorted)
        m._hash, m._row64, m._col64, m._csr = self._hash, self._row64, self._col64, self._csr
        m._order, m._tstruct = self._order, self._tstruct
        return m

    # ------------------------------------------------------------ CSR view
    def _csr_structure(self):
        """(row_ptr int64, col int32, perm or None, block) on the values' device.

        Matrices whose (block) rows are sorted -- every assembler output and
        every condensed matrix -- need no permutation."""
        if self._csr is not None:
            return self._csr
        dev = self.values.device
        H = self._block
        if H > 1:
            br, bc = self._block_row.to(dev).long(), self._block_col.to(dev).long()
            n = self.shape[0] // H
        else:
            br, bc = self._row_src.to(dev).long(), self._col_src.to(dev).long()
            n = self.shape[0]
        key = br * self.shape[1] + bc
        perm = None
        if self._sorted is not True:
            if key.numel() > 1 and not bool((key[1:] >= key[:-1]).all()):
                perm = torch.argsort(key, stable=True)
                br, bc = br[perm], bc[perm]
        if self._topology is not None and H == 1 and perm is None:
            rp = self._topology.row_ptr(dev)
        else:
            counts = torch.bincount(br, minlength=n)
            rp = torch.zeros(n + 1, dtype=torch.int64, device=dev)
            torch.cumsum(counts, 0, out=rp[1:])
        self._csr = (rp, bc.to(torch.int32).contiguous(), perm, H)
        return self._csr

    def _row_order(self) -> torch.Tensor:
        """int32 [n_rows] on the values' device: the (block) rows by
        decreasing length, ties in row order (computed once, on the host)."""
        if self._order is None:
            rp = self._csr_structure()[0]
            lens = np.diff(rp.cpu().numpy())
            order = np.argsort(-lens, kind="stable").astype(np.int32)
            self._order = torch.from_numpy(order).to(rp.device)
        return self._order

    def matvec(self, x: torch.Tensor, out: Optional[torch.Tensor] = None, alpha: float = 1.0,
               beta: float = 0.0) -> torch.Tensor:
        """A x (``out = alpha A x + beta out`` with ``out``).  Without ``out``
        the product is differentiable in the values and in x, as the
        reference's torch sparse product is: dL/dx = A^T dL/dy and dL/dA_ij =
        dL/dy_i x_j."""
        from .solve import spmv
        if out is None and alpha == 1.0 and torch.is_grad_enabled() and (
                self.values.requires_grad or (torch.is_tensor(x) and x.requires_grad)):
            return _SparseMatVec.apply(self.values, x, self)
        return spmv(self, x, out=out, alpha=alpha, beta=beta)

    def __matmul__(self, x: torch.Tensor) -> torch.Tensor:
        if x.dim() == 1:
            return self.matvec(x)
        return torch.stack([self.matvec(x[:, j].contiguous()) for j in range(x.shape[1])], 1)

    # ------------------------------------------------------------ arithmetic
    # (the reference's SparseMatrix inherits them from torch-sla's sparse
    # tensor: time integrators write M + dt * K); differentiable in the values
    def _same_layout(self, other: "SparseMatrix") -> bool:
        if self.shape != other.shape or self._block != other._block or self.nnz != other.nnz:
            return False
        if self._topology is not None and self._topology is other._topology:
            return True
        if self._row_src is other._row_src and self._col_src is other._col_src:
            return True
        return self.layout_hash == other.layout_hash

    def __mul__(self, s) -> "SparseMatrix":
        if isinstance(s, SparseMatrix) or (torch.is_tensor(s) and s.numel() != 1):
            return NotImplemented
        return self.with_values(self.values * s)

    __rmul__ = __mul__

    def __truediv__(self, s) -> "SparseMatrix":
        if isinstance(s, SparseMatrix) or (torch.is_tensor(s) and s.numel() != 1):
            return NotImplemented
        return self.with_values(self.values / s)

    def __neg__(self) -> "SparseMatrix":
        return self.with_values(-self.values)

    def __add__(self, other) -> "SparseMatrix":
        if not isinstance(other, SparseMatrix):
            return NotImplemented
        if self.shape != other.shape:
            raise ValueError(f"cannot add sparse matrices of shapes {self.shape} and {other.shape}")
        if self._same_layout(other):
            return self.with_values(self.values + other.values.to(self.values.dtype))
        # different patterns: the union, entries summed (scalar COO, row-major)
        dev = self.values.device
        row = torch.cat([self.row_indices.to(dev), other.row_indices.to(dev)])
        col = torch.cat([self.col_indices.to(dev), other.col_indices.to(dev)])
        val = torch.cat([self.values.reshape(-1), other.values.to(dev, self.values.dtype).reshape(-1)])
        key = row * self.shape[1] + col
        uniq, inv = torch.unique(key, sorted=True, return_inverse=True)
        out = torch.zeros(uniq.numel(), dtype=val.dtype, device=dev).index_add(0, inv, val)
        return SparseMatrix(out, uniq // self.shape[1], uniq % self.shape[1], self.shape, _sorted=True)

    def __sub__(self, other) -> "SparseMatrix":
        if not isinstance(other, SparseMatrix):
            return NotImplemented
        return self + (-other)

    # the dtype / device conversions of a torch tensor (the reference's
    # SparseMatrix is one), on the values; the layout is shared
    def to(self, *args, **kwargs) -> "SparseMatrix":
        v = self.values.to(*args, **kwargs)
        if v.device != self.values.device:
            m = SparseMatrix(v, self._row_src.to(v.device), self._col_src.to(v.device), self.shape,
                             _topology=self._topology, _block=self._block,
                             _block_row=None if self._block_row is None else self._block_row.to(v.device),
                             _block_col=None if self._block_col is None else self._block_col.to(v.device),
                             _sorted=self._sorted)
            m._hash = self._hash
            return m
        return self if v is self.values else self.with_values(v)

    def double(self) -> "SparseMatrix":
        return self.to(torch.float64)

    def float(self) -> "SparseMatrix":
        return self.to(torch.float32)

    def transpose(self) -> "SparseMatrix":
        """A^T with the same values array (entry k of A is entry k of A^T;
        its CSR view orders them when it is built, once per layout)."""
        if self._block > 1:
            H = self._block
            vals = self.values.reshape(-1, H, H).transpose(1, 2).reshape(-1)
            m = SparseMatrix(vals, self._col_src, self._row_src, (self.shape[1], self.shape[0]), _block=H,
                             _block_row=self._block_col, _block_col=self._block_row, _sorted=False)
        else:
            m = SparseMatrix(self.values, self.col_indices, self.row_indices, (self.shape[1], self.shape[0]),
                             _sorted=False)
        key = str(self.values.device)
        hold = self._tstruct.get(key)
        if hold is None:
            m._csr_structure()
            m._row_order()
            self._tstruct[key] = (m._csr, m._order)
        else:
            m._csr, m._order = hold
        return m

    @property
    def T(self) -> "SparseMatrix":
        return self.transpose()

    # direct methods of the inherited solve (torch-sla); here iterative
    # solves to a tight tolerance stand in for them
    _DIRECT = ("lu", "cholesky", "ldlt", "umfpack", "superlu", "direct", "qr")
    _DIRECT_BACKENDS = ("scipy", "cudss", "cupy", "eigen", "petsc")

    def solve(self, b: torch.Tensor, method: Optional[str] = None, **kwargs) -> torch.Tensor:
        """x = A^-1 b on the GPU: "cg" (Jacobi-PCG, A symmetric positive
        definite; keyword arguments of ``pcg_solve``) or "bicgstab"
        (Jacobi-BiCGSTAB, any square A; keyword arguments of
        ``bicgstab_solve``); differentiable in the values and in b (the
        adjoint solves with A^T).

        The keywords of the solve the reference's SparseMatrix inherits
        (torch-sla: ``backend``, ``method``, ``preconditioner``, ``tol``,
        ``atol``, ``max_iter``, ``x0``, ``is_spd``, ``verbose``) are
        accepted: the kernels of this library run on the matrix's device
        whatever the ``backend``, the preconditioner is Jacobi, ``tol`` is
        the relative residual, and a direct method or ``method=None``
        selects CG for an SPD matrix (``is_spd``, default True) and BiCGSTAB
        otherwise; a direct method, or no method with a backend whose
        default is direct (``"scipy"``, ``"cudss"``, ...), solves to a
        relative residual of 1e-12 unless ``tol`` says otherwise."""
        kw = dict(kwargs)
        backend = str(kw.pop("backend", "auto") or "auto").lower()
        kw.pop("verbose", None)
        kw.pop("preconditioner", None)
        is_spd = bool(kw.pop("is_spd", True))
        tol = kw.pop("tol", None)
        m = (method or "auto").lower()
        # a direct method, or a backend whose default is one, asks for a
        # solution accurate to rounding
        direct = m in self._DIRECT or (method is None and backend in self._DIRECT_BACKENDS)
        if m in ("auto", "default") or direct:
            m = "cg" if is_spd else "bicgstab"
        if m not in ("cg", "bicgstab"):
            raise ValueError(f"solve: method must be 'cg', 'bicgstab', a direct method or None, not {method!r}")
        if tol is None and direct and "rtol" not in kw and "atol" not in kw:
            tol = 1e-12
        if tol is not None:
            kw["rtol"] = float(tol)
            if m == "bicgstab":
                kw.setdefault("atol", 0.0)
        if m == "cg":
            kw.pop("atol", None)
        if torch.is_grad_enabled() and (self.values.requires_grad or b.requires_grad):
            from .adjoint import SparseSolve
            return SparseSolve.apply(self.values, b, self, dict(kw, method=m))
        from .solve import bicgstab_solve, pcg_solve
        return (pcg_solve if m == "cg" else bicgstab_solve)(self, b, **kw)

    def __repr__(self):
        return (f"SparseMatrix(shape={self.shape}, nnz={self.nnz}, dtype={self.dtype}, "
                f"device={self.device}{', block=%d' % self._block if self._block > 1 else ''})")


class _SparseMatVec(torch.autograd.Function):
    """y = A x through the SpMV kernel, differentiable in A's values and in
    x: dL/dx = A^T g (the transpose's own CSR view, built once per layout),
    dL/dvalues = g_row x_col per stored entry (per block entry, g of the
    block's rows times x of its columns, for block matrices)."""

    @staticmethod
    def forward(ctx, values, x, A):
        from .solve import spmv
        ctx.A = A
        ctx.x_dtype = x.dtype
        ctx.save_for_backward(x)
        return spmv(A, x.detach())

    @staticmethod
    def backward(ctx, g):
        from .solve import spmv
        (x,) = ctx.saved_tensors
        A = ctx.A
        g = g.to(A.values.dtype).contiguous()
        gv = gx = None
        if ctx.needs_input_grad[1]:
            gx = spmv(A.transpose(), g).to(ctx.x_dtype)
        if ctx.needs_input_grad[0]:
            xd = x.detach().to(device=g.device, dtype=g.dtype)
            H = A._block
            if H > 1:
                br = A._block_row.to(g.device).long()
                bc = A._block_col.to(g.device).long()
                gv = g.view(-1, H)[br][:, :, None] * xd.reshape(-1, H)[bc][:, None, :]
            else:
                gv = g[A._row_src.to(g.device).long()] * xd[A._col_src.to(g.device).long()]
            gv = gv.reshape(A.values.shape)
        return gv, gx, None
