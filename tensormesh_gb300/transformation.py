"""``Transformation`` and the two projectors, with the reference's interfaces.

* ``Transformation(points, elements, element_type, quadrature_order)``
  (element/transformation.py:9-1276): quadrature, ``shape_val`` [Q,B],
  ``shape_grad`` [E,Q,B,D], ``JxW`` [E,Q], ``batch_shape_val``,
  ``batch_shape_grad_jxw``.  Gradients and JxW come from the
  ``tm_shape_grad_jxw`` kernel and are recomputed from the current points on
  every access (the reference caches them on first access and does not
  invalidate the cache in ``update_points``, :137-161).
* ``ReduceProjector(indices, from_shape, to_shape)`` (assemble/projector.py:24-129)
  and ``SparseProjector(from_, to_, from_shape, to_shape)`` (:131-248): both
  compute out[to] = sum of x[from] with the deterministic
  ``tm_project_reduce`` kernel over the inverse index map.
"""
from typing import Optional, Sequence, Union

import numpy as np
import torch
import torch.nn as nn

from . import _lib
from .element import element_info, element_tables, packed_tables


class Transformation(nn.Module):
    def __init__(self, points: torch.Tensor, elements: torch.Tensor, element_type: str,
                 quadrature_order: int = 2):
        super().__init__()
        self.info = element_info(element_type)
        self.element_type = element_type
        self.basis_order = self.info.order
        self.quadrature_order = quadrature_order
        self.register_buffer("elements", elements)
        self.update_points(points)

    def update_points(self, points: torch.Tensor):
        self.register_buffer("points", points)
        self.n_points = int(points.shape[0])

    @property
    def dim(self) -> int:
        return int(self.points.shape[-1])

    @property
    def device(self):
        return self.points.device

    @property
    def dtype(self):
        return self.points.dtype

    @property
    def n_elements(self) -> int:
        return int(self.elements.shape[0])

    @property
    def n_basis(self) -> int:
        return self.info.n_basis

    @property
    def element_coords(self) -> torch.Tensor:
        return self.points[self.elements]

    @property
    def quadrature(self):
        t = element_tables(self.element_type, self.quadrature_order)
        return (torch.tensor(t["w"], dtype=self.dtype, device=self.device),
                torch.tensor(t["xi"], dtype=self.dtype, device=self.device))

    @property
    def n_quadrature(self) -> int:
        return len(element_tables(self.element_type, self.quadrature_order)["w"])

    @property
    def shape_val(self) -> torch.Tensor:
        t = element_tables(self.element_type, self.quadrature_order)
        return torch.tensor(t["phi"], dtype=self.dtype, device=self.device)

    def _geometry(self):
        _lib.require_cuda(self.points, "points")
        lib = _lib.load()
        dev = self.points.device
        E, Q, B, D = self.n_elements, self.n_quadrature, self.n_basis, self.dim
        pts = self.points.detach().to(torch.float64).contiguous()
        conn = self.elements.to(device=dev, dtype=torch.int32).contiguous()
        tables = torch.from_numpy(packed_tables(self.element_type, self.quadrature_order)).to(dev)
        tb = _lib.ElementTables(self.info.code, Q, _lib.ptr(tables))
        grad = torch.empty(E, Q, B, D, dtype=torch.float64, device=dev)
        jxw = torch.empty(E, Q, dtype=torch.float64, device=dev)
        _lib.check(lib.tm_shape_grad_jxw(E, _lib.ptr(conn), _lib.ptr(pts), tb, _lib.ptr(grad), _lib.ptr(jxw),
                                         _lib.stream_handle(dev)), "tm_shape_grad_jxw")
        return grad.to(self.dtype), jxw.to(self.dtype)

    @property
    def shape_grad(self) -> torch.Tensor:
        return self._geometry()[0]

    @property
    def JxW(self) -> torch.Tensor:
        return self._geometry()[1]

    def batch_shape_val(self, start: int, batch: int) -> torch.Tensor:
        sv = self.shape_val
        return sv[start:] if batch in (-1, None) else sv[start:start + batch]

    def batch_shape_grad_jxw(self, element_start: int = 0, element_batch: int = -1,
                             quadrature_start: int = 0, quadrature_batch: int = -1):
        g, j = self._geometry()
        es = slice(element_start, None if element_batch in (-1, None) else element_start + element_batch)
        qs = slice(quadrature_start, None if quadrature_batch in (-1, None) else quadrature_start + quadrature_batch)
        return g[es, qs], j[es, qs]


Shape = Union[Sequence[int], int, np.ndarray, torch.Size]


def _shape(s) -> tuple:
    if isinstance(s, int):
        return (s,)
    return tuple(int(v) for v in s)


class _DeterministicScatter(nn.Module):
    """out[t] = sum over the sources mapped to t, in source order.  The
    inverse index map (sources sorted by target) is built on first use."""

    _src = None
    _seg = None

    def _build_inverse(self):
        d = self.indices.detach().cpu().numpy().astype(np.int64)
        order = np.argsort(d, kind="stable")
        seg = np.zeros(self._to_size + 1, dtype=np.int64)
        np.cumsum(np.bincount(d, minlength=self._to_size), out=seg[1:])
        self._src = torch.from_numpy(order)
        self._seg = torch.from_numpy(seg)

    def _scatter(self, x: torch.Tensor) -> torch.Tensor:
        if self._src is None:
            self._build_inverse()
        _lib.require_cuda(x, "projector input")
        lib = _lib.load()
        assert tuple(x.shape[:len(self.from_shape)]) == tuple(self.from_shape), \
            f"the shape of x must be [{self.from_shape}, ...], but got {tuple(x.shape)}"
        dim_shape = x.shape[len(self.from_shape):]
        width = int(np.prod(dim_shape)) if len(dim_shape) else 1
        xs = x.reshape(self._from_size, width).contiguous()
        out = torch.empty(self._to_size, width, dtype=x.dtype, device=x.device)
        seg, src = self._seg.to(x.device), self._src.to(x.device)
        _lib.check(lib.tm_project_reduce(_lib.dtype_code(x.dtype), self._to_size, width, _lib.ptr(seg),
                                         _lib.ptr(src), _lib.ptr(xs), _lib.ptr(out), _lib.stream_handle(x.device)),
                   "tm_project_reduce")
        return out.reshape(*self.to_shape, *dim_shape)


class ReduceProjector(_DeterministicScatter):
    def __init__(self, indices, from_shape: Shape, to_shape: Shape, use_fp64: bool = False):
        super().__init__()
        if isinstance(indices, np.ndarray):
            indices = torch.from_numpy(indices)
        assert indices.dim() == 1, f"indices must be 1D, but got {indices.dim()}"
        self.register_buffer("indices", indices)
        self.from_shape, self.to_shape = _shape(from_shape), _shape(to_shape)
        self.use_fp64 = use_fp64
        self._from_size = int(np.prod(self.from_shape))
        self._to_size = int(np.prod(self.to_shape))

    @property
    def device(self):
        return self.indices.device

    def __call__(self, x: torch.Tensor) -> torch.Tensor:
        if self.use_fp64 and x.dtype != torch.float64:
            return self._scatter(x.double()).to(x.dtype)
        return self._scatter(x)

    def __repr__(self):
        return f"ReduceProjector({self.from_shape} -> {self.to_shape}, device={self.device})"


class SparseProjector(_DeterministicScatter):
    def __init__(self, from_, to_, from_shape: Shape, to_shape: Shape, dtype=None):
        super().__init__()
        if isinstance(from_, np.ndarray):
            from_ = torch.from_numpy(from_)
        if isinstance(to_, np.ndarray):
            to_ = torch.from_numpy(to_)
        assert from_.shape == to_.shape and from_.dim() == 1
        self.from_shape, self.to_shape = _shape(from_shape), _shape(to_shape)
        self._from_size = int(np.prod(self.from_shape))
        self._to_size = int(np.prod(self.to_shape))
        # a (from, to) pair listed k times contributes k times, as in the 0/1 matrix
        f, t = from_.cpu().long().numpy(), to_.cpu().long().numpy()
        order = np.lexsort((f, t))
        seg = np.zeros(self._to_size + 1, dtype=np.int64)
        np.cumsum(np.bincount(t, minlength=self._to_size), out=seg[1:])
        self._src = torch.from_numpy(f[order].copy())
        self._seg = torch.from_numpy(seg)
        self.register_buffer("from_", from_.long())
        self.register_buffer("to_", to_.long())

    @property
    def device(self):
        return self.from_.device

    def __call__(self, x: torch.Tensor) -> torch.Tensor:
        return self._scatter(x)

    def __repr__(self):
        return f"SparseProjector({self.from_shape} -> {self.to_shape}, device={self.device})"
