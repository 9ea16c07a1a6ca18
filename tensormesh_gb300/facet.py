"""Boundary-facet assembly with the reference's interface
(assemble/facet_assembler.py:17-567): ``FacetAssembler.from_mesh(mesh,
boundary_mask=None, quadrature_order=2, project='reduce')``,
``from_elements``, ``from_assembler`` and ``__call__(points=None, func=None,
point_data=None)`` returning the flattened nodal vector [N] or [N*H].

A facet (edge of a triangle, face of a tetrahedron) of an element is selected
when all of its nodes are boundary nodes, element by element, as the
reference selects them (facet_assembler.py:447-466); each selected
(element, facet) pair is one item, integrated by ``tm_assemble_facet_vector``
with the facet's own basis (the element basis restricted to the facet) and
reduced into the nodes by a node chunk plan, deterministically.

The reference's integrand is a Python ``forward`` evaluated by vmap; here the
load forms it is used for are built in: ``const_facet_assembler(c)``
(``c * v``, c a scalar or a traction vector), ``LoadFacetAssembler``
(``f * v``, f nodal in point_data, [N] or [N, H]) and
``func_facet_assembler(g)`` (``g(x) * v``, g evaluated on the device at the
facet quadrature points).  Any other ``forward`` raises NotImplementedError.
"""
import ctypes as C
from typing import Callable, Dict, Optional

import numpy as np
import torch
import torch.nn as nn

from . import _lib
from .element import facet_info, facet_tables, packed_facet_tables
from .plan import DevicePlan, HostPlan

FACET_CHUNK = 256


class FacetAssembler(nn.Module):
    """Integrate a built-in load form over the selected boundary facets."""

    _tm_facet_form = None       # ("const", c) | ("nodal", key) | ("func", g) on the built-ins

    def __init__(self, items: np.ndarray, element_type: str, n_points: int, quadrature_order: int,
                 points: torch.Tensor, *args, **kwargs):
        super().__init__()
        self.element_types = [element_type]
        self.element_type = element_type
        self.n_points = int(n_points)
        self.quadrature_order = int(quadrature_order)
        self.dimension = int(points.shape[1])
        self.items = items                       # [n_items, Bf] facet nodes, item order
        self._points = points
        self._plans: Dict = {}
        self._tables: Dict = {}
        self.__post_init__(*args, **kwargs)

    def __post_init__(self, *args, **kwargs):
        pass

    def forward(self, *args):
        raise NotImplementedError(
            "tensormesh_gb300 assembles the built-in facet load forms (const_facet_assembler, "
            "LoadFacetAssembler, func_facet_assembler); custom Python integrands are not supported")

    # ------------------------------------------------------------ builders
    @staticmethod
    def _select(conn: np.ndarray, boundary: np.ndarray, element_type: str) -> np.ndarray:
        """Facet nodes of every (element, facet) pair whose nodes are all
        boundary nodes, element-major (facet_assembler.py:447-466)."""
        fi = facet_info(element_type)
        nodes = np.array(fi.nodes)                                   # [n_facet, Bf]
        fnodes = conn[:, nodes]                                      # [E, n_facet, Bf]
        sel = boundary[fnodes].all(-1)                               # [E, n_facet]
        return np.ascontiguousarray(fnodes[sel], dtype=np.int64)     # row-major = element, then facet

    @classmethod
    def from_elements(cls, points: torch.Tensor, elements: Dict[str, torch.Tensor], boundary_mask: torch.Tensor,
                      quadrature_order: int = 2, device="cpu", dtype: torch.dtype = torch.float32,
                      project: str = "reduce", *args, **kwargs):
        if project not in ("reduce", "sparse"):
            raise ValueError(f"project should be either 'reduce' or 'sparse', but got {project}")
        if len(elements) != 1:
            raise NotImplementedError("a FacetAssembler here holds one element type")
        (etype, conn), = elements.items()
        conn_np = conn.detach().cpu().numpy().astype(np.int64)
        bnd = boundary_mask.detach().cpu().numpy().astype(bool)
        items = cls._select(conn_np, bnd, etype)
        pts = points.detach().to(device=device, dtype=dtype)
        return cls(items, etype, points.shape[0], quadrature_order, pts, *args, **kwargs)

    @classmethod
    def from_mesh(cls, mesh, boundary_mask=None, quadrature_order: int = 2, project: str = "reduce",
                  *args, **kwargs):
        if boundary_mask is None:
            bnd = mesh.boundary_mask
        elif isinstance(boundary_mask, str):
            bnd = mesh.point_data[boundary_mask]
        else:
            bnd = boundary_mask
        assert bnd.dtype == torch.bool and bnd.dim() == 1 and bnd.shape[0] == mesh.n_points, \
            "boundary_mask must be a 1D bool tensor of length n_points"
        et = mesh.default_element_type
        return cls.from_elements(mesh.points, {et: mesh.elements()}, bnd, quadrature_order,
                                 mesh.points.device, mesh.points.dtype, project, *args, **kwargs)

    @classmethod
    def from_assembler(cls, obj: "FacetAssembler", *args, **kwargs):
        return cls(obj.items, obj.element_type, obj.n_points, obj.quadrature_order, obj._points, *args, **kwargs)

    @property
    def n_items(self) -> int:
        return int(self.items.shape[0])

    def _plan(self, device: torch.device) -> DevicePlan:
        if device not in self._plans:
            fi = facet_info(self.element_type)
            host = HostPlan(self.items.reshape(-1, fi.n_basis), self.n_points, _lib.TM_PLAN_KIND_NODE,
                            FACET_CHUNK)
            self._plans[device] = DevicePlan(host, device)
        return self._plans[device]

    def _table_struct(self, device: torch.device):
        if device not in self._tables:
            packed = torch.from_numpy(packed_facet_tables(self.element_type, self.quadrature_order)).to(device)
            t = _lib.FacetTables()
            t.facet_type = facet_info(self.element_type).code
            t.n_quad = len(facet_tables(self.element_type, self.quadrature_order)["w"])
            t.packed = _lib.ptr(packed)
            self._tables[device] = (t, packed)
        return self._tables[device][0]

    def quadrature_points(self, points: torch.Tensor) -> torch.Tensor:
        """Physical coordinates of the facet quadrature points [n_items, Q, D]."""
        psi = torch.from_numpy(facet_tables(self.element_type, self.quadrature_order)["psi"]).to(
            device=points.device, dtype=points.dtype)
        items = torch.from_numpy(self.items).to(points.device)
        return torch.einsum("qb,fbd->fqd", psi, points[items])

    # --------------------------------------------------------------- call
    def __call__(self, points: Optional[torch.Tensor] = None, func: Optional[Callable] = None,
                 point_data: Optional[Dict[str, torch.Tensor]] = None) -> torch.Tensor:
        point_data = dict(point_data or {})
        if points is None:
            points = self._points
        _lib.require_cuda(points, "points")
        for key, value in point_data.items():
            assert value.shape[0] == self.n_points, \
                f"the shape of {key} should be [n_point, ...], but got {tuple(value.shape)}"
        form = self._tm_facet_form
        if func is not None:
            raise NotImplementedError("tensormesh_gb300 does not evaluate custom Python facet integrands (func=); "
                                      "use const_facet_assembler, LoadFacetAssembler or func_facet_assembler")
        if form is None:
            self.forward()                       # raises: no built-in form
        dev, dt = points.device, points.dtype
        kind, arg = form
        # the source as a tensor: constant [W], nodal [N, W] or per point
        # [items, Q, W] (a function of the points' quadrature coordinates)
        if kind == "const":
            src = arg if torch.is_tensor(arg) else torch.as_tensor(arg, dtype=torch.float64)
            src = src.reshape(-1)
        elif kind == "nodal":
            f = point_data[arg].to(device=dev, dtype=dt)
            src = f.reshape(self.n_points, -1)
        else:
            grad_x = torch.is_grad_enabled() and points.requires_grad
            xq = self.quadrature_points(points if grad_x else points.detach())
            src = torch.as_tensor(arg(xq), device=dev, dtype=dt)
            src = src.reshape(self.n_items, xq.shape[1], -1)
        if torch.is_grad_enabled() and (points.requires_grad or src.requires_grad):
            return FacetLoad.apply(points, src, self, kind)
        return self._run(points.detach(), kind, src.detach())

    def _args(self, pts: torch.Tensor, kind: str, src: torch.Tensor):
        dev, dt = pts.device, pts.dtype
        a = _lib.FacetVectorArgs()
        a.dtype = _lib.dtype_code(dt)
        a.n_points = self.n_points
        a.points = _lib.ptr(pts)
        keep = [pts]
        if kind == "const":
            c = src.detach().to(torch.float64).reshape(-1)
            if c.numel() > 3:
                raise ValueError("a constant facet load has 1..3 components")
            a.source, a.width = _lib.TM_SOURCE_CONST, c.numel()
            for i in range(c.numel()):
                a.const_value[i] = float(c[i])
        elif kind == "nodal":
            f2 = src.detach().to(device=dev, dtype=dt).contiguous()
            a.source, a.width, a.values = _lib.TM_SOURCE_NODAL, f2.shape[1], _lib.ptr(f2)
            keep.append(f2)
        else:
            g2 = src.detach().to(device=dev, dtype=dt).contiguous()
            a.source, a.width, a.values = _lib.TM_SOURCE_QUAD, g2.shape[2], _lib.ptr(g2)
            keep.append(g2)
        if not 1 <= a.width <= 3:
            raise ValueError(f"facet loads have 1..3 components, got {a.width}")
        a.plan = self._plan(dev).struct()
        a.tables = self._table_struct(dev)
        return a, keep

    def _run(self, pts: torch.Tensor, kind: str, src: torch.Tensor) -> torch.Tensor:
        dev, dt = pts.device, pts.dtype
        pts = pts.contiguous()
        a, keep = self._args(pts, kind, src)
        lib = _lib.load()
        ws = torch.empty(max(1, lib.tm_facet_vector_workspace_bytes(C.byref(a))), dtype=torch.uint8, device=dev)
        out = torch.empty(self.n_points, a.width, dtype=dt, device=dev)
        a.workspace, a.out = _lib.ptr(ws), _lib.ptr(out)
        _lib.check(lib.tm_assemble_facet_vector(C.byref(a), _lib.stream_handle(dev)), "tm_assemble_facet_vector")
        return out.reshape(-1)


class FacetLoad(torch.autograd.Function):
    """A facet load vector as a function of the node coordinates and of its
    source (constant [W], nodal [N, W] or per point [items, Q, W]): the
    backward runs ``tm_facet_adjoint`` (the points through the facet
    measure; dL/dvalues of a per-point source) and, for constant and nodal
    sources, the forward kernel (dL/dc_w = lam_w . b(c = 1); dL/df = the
    facet load of the nodal source lam)."""

    @staticmethod
    def forward(ctx, points, src, fa, kind):
        ctx.fa, ctx.kind = fa, kind
        ctx.save_for_backward(points, src)
        return fa._run(points.detach(), kind, src.detach())

    @staticmethod
    def backward(ctx, gb):
        points, src = ctx.saved_tensors
        fa, kind = ctx.fa, ctx.kind
        dev = gb.device
        pts = points.detach().to(torch.float64).contiguous()
        s64 = src.detach().to(device=dev, dtype=torch.float64)
        W = (s64.numel() if kind == "const" else s64.shape[-1])
        lam = gb.detach().to(torch.float64).reshape(fa.n_points, W).contiguous()
        gp = gs = None
        want_q = kind == "func" and ctx.needs_input_grad[1]
        if ctx.needs_input_grad[0] or want_q:
            base, keep = fa._args(pts, kind, s64)
            a = _lib.FacetAdjointArgs()
            a.base = base
            a.lam = _lib.ptr(lam)
            D = points.shape[1]
            gpts = torch.empty(fa.n_points, D, dtype=torch.float64, device=dev) if ctx.needs_input_grad[0] else None
            # (contiguous: the kernel writes [items, Q, W] in order, whatever
            # the source's strides)
            gq = torch.empty(s64.shape, dtype=torch.float64, device=dev) if want_q else None
            a.grad_points, a.grad_values = _lib.ptr(gpts), _lib.ptr(gq)
            lib = _lib.load()
            ws = torch.empty(max(1, lib.tm_facet_adjoint_workspace_bytes(C.byref(a))), dtype=torch.uint8, device=dev)
            a.base.workspace = _lib.ptr(ws)
            _lib.check(lib.tm_facet_adjoint(C.byref(a), _lib.stream_handle(dev)), "tm_facet_adjoint")
            if gpts is not None:
                gp = gpts.to(points.dtype)
            if gq is not None:
                gs = gq.to(src.dtype)
        if ctx.needs_input_grad[1] and kind == "const":
            b1 = fa._run(pts, "const", torch.ones(W, dtype=torch.float64)).reshape(fa.n_points, W)
            gs = (lam * b1).sum(0).reshape(src.shape).to(device=src.device, dtype=src.dtype)
        elif ctx.needs_input_grad[1] and kind == "nodal":
            gs = fa._run(pts, "nodal", lam).reshape(src.shape).to(src.dtype)
        return gp, gs, None, None


def const_facet_assembler(c=1):
    """``c * v`` over the selected facets; ``c`` a scalar or a vector
    (a constant traction)."""
    class ConstFacetAssembler(FacetAssembler):
        def __post_init__(self, c=c):
            self.c = c

        def forward(self, v):
            return self.c * v

        @property
        def _tm_facet_form(self):
            return ("const", self.c)

    return ConstFacetAssembler


def func_facet_assembler(g: Callable = lambda x: x[..., 0]):
    """``g(x) * v`` over the selected facets, g a function of the facet
    quadrature points' coordinates [..., D] returning [...] or [..., H]."""
    class FuncFacetAssembler(FacetAssembler):
        def __post_init__(self, g=g):
            self.g = g

        def forward(self, v, x):
            return self.g(x) * v

        @property
        def _tm_facet_form(self):
            return ("func", self.g)

    return FuncFacetAssembler


class LoadFacetAssembler(FacetAssembler):
    """``f * v`` over the selected facets, f given at the nodes
    (point_data["f"], [N] or [N, H])."""

    _tm_facet_form = ("nodal", "f")

    def forward(self, v, f):
        return f * v
