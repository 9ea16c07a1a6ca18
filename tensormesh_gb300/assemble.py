"""``ElementAssembler`` and ``NodeAssembler`` with the reference's interfaces
(assemble/element_assembler.py, assemble/node_assembler.py), running the
fused GPU kernels of ``libtmgb300.so``.

The reference lifts a Python ``forward`` integrand over elements,
quadrature points and basis pairs with nested ``vmap`` and scatters with
``index_add_``.  Here each built-in family is one kernel (see
``csrc/tm_assemble.cu``); the class of the assembler selects it.  Calling an
assembler whose ``forward`` is a custom Python integrand raises
``NotImplementedError`` -- there is no CPU or vmap path.

Linear forms are the exception that is kept general: any ``NodeAssembler``
whose ``forward`` is a source term times the test function, ``g(x, data) * v``
(the shape of every load form in the reference's documentation), is assembled
by evaluating ``g`` on the device at the quadrature points (``forward`` called
once with ``v = 1`` on [E, Q]-batched arguments, as the reference's own
broadcast fast path does, node_assembler.py:173-240) and integrating and
reducing it with the kernel.
"""
import inspect
import math
from typing import Callable, Dict, Mapping, Optional, Union

import numpy as np
import torch
import torch.nn as nn

from . import _lib
from .element import element_info, element_tables, element_type2dimension
from .plan import MixedTopology, Topology
from .sparse import SparseMatrix
from .transformation import ReduceProjector, SparseProjector, Transformation


class BufferDict(nn.Module):
    """Named buffers that follow ``.to()`` (the reference's nn.BufferDict)."""

    def __init__(self, d: Optional[Mapping[str, torch.Tensor]] = None):
        super().__init__()
        self._keys = []
        for k, v in (d or {}).items():
            self[k] = v

    def __setitem__(self, k, v):
        if k not in self._keys:
            self._keys.append(k)
        self.register_buffer(k, v)

    def __getitem__(self, k):
        return getattr(self, k)

    def __contains__(self, k):
        return k in self._keys

    def __iter__(self):
        return iter(self._keys)

    def __len__(self):
        return len(self._keys)

    def keys(self):
        return list(self._keys)

    def values(self):
        return [self[k] for k in self._keys]

    def items(self):
        return [(k, self[k]) for k in self._keys]


def _single_type(elements) -> tuple:
    if isinstance(elements, torch.Tensor):
        raise TypeError("elements must be a {element_type: tensor} mapping")
    keys = list(elements.keys())
    if len(keys) != 1:
        raise NotImplementedError(f"mixed-element meshes ({keys}) are not assembled by tensormesh_gb300")
    element_info(keys[0])
    return keys[0], elements[keys[0]]


def _mesh_elements(mesh) -> Dict[str, torch.Tensor]:
    elements = mesh.elements()
    if isinstance(elements, torch.Tensor):
        elements = {mesh.default_element_type: elements}
    return dict(elements)


class _AssemblerBase(nn.Module):
    _topology: Optional[Topology] = None

    def type(self, dtype: torch.dtype):
        if dtype == torch.float64:
            self.double()
        elif dtype == torch.float32:
            self.float()
        else:
            raise Exception(f"the dtype {dtype} is not supported")
        return self

    @property
    def device(self) -> torch.device:
        return next(iter(self.transformation.values())).device

    @property
    def dtype(self) -> torch.dtype:
        return next(iter(self.transformation.values())).dtype

    def _topo(self, matrix: bool) -> Topology:
        if self._topology is None:
            et = self.element_types[0]
            trans = self.transformation[et]
            self._topology = Topology(trans.points, self.elements[et], et, trans.quadrature_order, matrix=matrix)
        return self._topology

    def __post_init__(self, *args, **kwargs):
        pass


# ============================================================================
# Recognition of user weak forms
# ============================================================================
class RecognisedForm:
    """A user ``forward`` identified as a built-in family: ``form`` is
    "diffusion", "mass" or "elasticity", ``coef`` the name of its coefficient
    argument (or None) and ``nu`` the Poisson ratio of an elasticity form.
    The family's modulus (kappa, rho or E) is ``scale * c`` for a form
    linear in its coefficient c, else ``cmap(c)``: the form evaluated per
    element on fixed probe arguments (``torch.func.vmap`` over c, as the
    reference vmaps ``forward``), differentiable in c."""

    def __init__(self, form: str, coef: Optional[str], nu: float = 0.3, scale: float = 1.0, cmap=None):
        self.form, self.coef, self.nu, self.scale, self.cmap = form, coef, nu, scale, cmap

    def modulus(self, c):
        """The family's modulus for the coefficient value(s) c."""
        if self.cmap is not None:
            return self.cmap(c)
        if self.scale == 1.0:
            return c
        return c * self.scale if torch.is_tensor(c) else float(c) * self.scale

    def __repr__(self):
        return (f"RecognisedForm({self.form!r}, coef={self.coef!r}, nu={self.nu}, scale={self.scale}, "
                f"nonlinear={self.cmap is not None})")


_FIELD_ARGS = ("gradu", "gradv", "u", "v", "x")
_MODULUS_KEY = "_tm_modulus"          # element data: a modulus derived from a per-node coefficient
_UNSET = object()


def _close(a: torch.Tensor, b: torch.Tensor, tol: float = 1e-12) -> bool:
    a, b = torch.as_tensor(a, dtype=torch.float64), torch.as_tensor(b, dtype=torch.float64)
    if a.shape != b.shape:
        return False
    return bool((a - b).abs().max() <= tol * max(1.0, float(b.abs().max())))


def recognise_form(asm) -> Optional[RecognisedForm]:
    """Identify the ``forward`` of an ``ElementAssembler`` subclass with one
    of the families the kernels assemble, the way the reference calls it
    (per element, quadrature point and basis pair, arguments bound by name:
    element_assembler.py:231-445): ``forward(gradu, gradv[, c])`` returning
    ``c * (gradu @ gradv)`` (diffusion, e.g. the ``SIMPLaplace`` form of
    examples/inverse_design/thermal_topology.py:48-52), ``forward(u, v[, c])``
    returning ``c * u * v`` (mass), or ``forward(gradu, gradv[, c])`` returning
    a D x D block ``c (lam gu gv^T + mu (gv gu^T + (gu . gv) I))`` (isotropic
    elasticity, ``Ba^T C Bb`` of builtin.py:168-178).  ``forward`` is probed
    on a few seeded random arguments in float64 and must reproduce the family
    to 1e-12 on each, with a coefficient that enters linearly; anything else
    (another argument, a nonlinear dependence) is a custom form (None).  The
    result is cached on the assembler (a form may read its own attributes,
    such as a Poisson ratio set by ``__post_init__``)."""
    cached = asm.__dict__.get("_tm_recognised", _UNSET)
    if cached is not _UNSET:
        return cached
    try:
        rec = _probe(asm)
    except Exception:
        rec = None
    asm.__dict__["_tm_recognised"] = rec
    return rec


def _probe(asm) -> Optional[RecognisedForm]:
    if type(asm).forward is ElementAssembler.forward:
        return None
    params = list(inspect.signature(asm.forward).parameters.values())
    if any(p.kind in (p.VAR_POSITIONAL, p.VAR_KEYWORD) for p in params):
        return None
    names = [p.name for p in params]
    coefs = [n for n in names if n not in _FIELD_ARGS]
    if len(coefs) > 1 or "x" in names:
        return None
    coef = coefs[0] if coefs else None
    fields = set(names) - set(coefs)
    D = asm.dimension
    g = torch.Generator().manual_seed(1234)
    draws = []
    for _ in range(3):
        c = 0.5 + float(torch.rand((), generator=g, dtype=torch.float64)) * 1.5
        draws.append((torch.randn(D, generator=g, dtype=torch.float64),
                      torch.randn(D, generator=g, dtype=torch.float64),
                      torch.randn((), generator=g, dtype=torch.float64),
                      torch.randn((), generator=g, dtype=torch.float64), c))

    def call(gu, gv, u, v, c):
        vals = {"gradu": gu, "gradv": gv, "u": u, "v": v}
        kw = {n: vals[n] for n in fields}
        if coef is not None:
            kw[coef] = torch.tensor(c, dtype=torch.float64)
        with torch.no_grad():
            return torch.as_tensor(asm.forward(**kw))

    def scalar_map(base_of):
        """s(c) per draw for out = s(c) base(args), checked on a second
        argument set at the same c; the linear scale or a per-element map."""
        svals = []
        for k, (gu, gv, u, v, c) in enumerate(draws):
            base = base_of(gu, gv, u, v)
            if abs(float(base)) < 1e-3:
                return None
            sk = float(call(gu, gv, u, v, c)) / float(base)
            gu2, gv2, u2, v2, _ = draws[(k + 1) % len(draws)]
            if not _close(call(gu2, gv2, u2, v2, c), sk * base_of(gu2, gv2, u2, v2)):
                return None
            svals.append((c, sk))
        return svals

    def make_cmap(evaluate):
        """c (a scalar or one value per element, on any device) -> the
        modulus, with autograd; the probe arguments follow c's device."""
        def cmap(c):
            ct = torch.as_tensor(c, dtype=torch.float64)
            ev = lambda ci: evaluate(ci, ct.device)
            if ct.dim() == 0:
                return ev(ct)
            return torch.func.vmap(ev)(ct.reshape(-1))
        return cmap

    def classify(svals, family, base0, extra=None):
        extra = extra or {}
        if coef is None:
            return RecognisedForm(family, None, scale=svals[0][1], **extra)
        ratios = [sk / c for c, sk in svals]
        if all(abs(r - ratios[0]) <= 1e-12 * max(1.0, abs(ratios[0])) for r in ratios):
            return RecognisedForm(family, coef, scale=ratios[0], **extra)
        return RecognisedForm(family, coef, cmap=make_cmap(base0), **extra)

    if fields == {"u", "v"}:
        svals = scalar_map(lambda gu, gv, u, v: u * v)
        if svals is None:
            return None
        gu0, gv0, u0, v0, _ = draws[0]

        def ev_mass(ci, dev):
            u, v = u0.to(dev), v0.to(dev)
            kw = {"u": u, "v": v}
            if coef:
                kw[coef] = ci
            return asm.forward(**kw) / (u * v)
        return classify(svals, "mass", ev_mass)
    if fields != {"gradu", "gradv"}:
        return None
    gu, gv, u, v, c = draws[0]
    out = call(gu, gv, u, v, c)
    if out.dim() == 0:
        svals = scalar_map(lambda gu, gv, u, v: gu @ gv)
        if svals is None:
            return None
        gu0, gv0 = draws[0][0], draws[0][1]

        def ev_diff(ci, dev):
            gu, gv = gu0.to(dev), gv0.to(dev)
            kw = {"gradu": gu, "gradv": gv}
            if coef:
                kw[coef] = ci
            return asm.forward(**kw) / (gu @ gv)
        return classify(svals, "diffusion", ev_diff)
    if tuple(out.shape) != (D, D):
        return None

    def basis(gu, gv):
        return torch.outer(gu, gv), torch.outer(gv, gu) + (gu @ gv) * torch.eye(D, dtype=torch.float64)

    # per draw: lam and mu of the block at that draw's coefficient (least
    # squares on its gradients), checked on a second gradient pair at the
    # same coefficient; lam / mu must be the same for every draw (one
    # Poisson ratio), and the modulus per unit coefficient linear or a map
    fits = []
    for k, (gu, gv, u, v, c) in enumerate(draws):
        a, b = basis(gu, gv)
        A = torch.stack([a.reshape(-1), b.reshape(-1)], 1)
        sol = torch.linalg.lstsq(A, call(gu, gv, u, v, c).reshape(-1, 1).to(torch.float64)).solution.reshape(-1)
        lam, mu = float(sol[0]), float(sol[1])
        if not (mu > 0 and lam + mu > 0):
            return None
        gu2, gv2 = draws[(k + 1) % len(draws)][:2]
        a2, b2 = basis(gu2, gv2)
        if not _close(call(gu2, gv2, u, v, c), lam * a2 + mu * b2):
            return None
        fits.append((c, lam, mu))
    if any(abs(l / m - fits[0][1] / fits[0][2]) > 1e-12 * max(1.0, abs(fits[0][1] / fits[0][2]))
           for _, l, m in fits):
        return None
    # the kernel's moduli: lam = E nu / ((1 + nu)(1 - 2 nu)), mu = E / (2 (1 + nu))
    lam0, mu0 = fits[0][1], fits[0][2]
    nu = lam0 / (2.0 * (lam0 + mu0))
    if not (-1.0 < nu < 0.5):
        return None
    svals = [(c, 2.0 * m * (1.0 + nu)) for c, _, m in fits]          # E at each draw
    gu0, gv0 = draws[0][0], draws[0][1]
    a0, b0 = basis(gu0, gv0)
    pinv = torch.linalg.pinv(torch.stack([a0.reshape(-1), b0.reshape(-1)], 1))

    def ev_el(ci, dev):
        kw = {"gradu": gu0.to(dev), "gradv": gv0.to(dev)}
        if coef:
            kw[coef] = ci
        return 2.0 * (1.0 + nu) * (pinv[1].to(dev) @ asm.forward(**kw).reshape(-1))
    return classify(svals, "elasticity", ev_el, {"nu": nu})


# ============================================================================
# Bilinear forms
# ============================================================================
class ElementAssembler(_AssemblerBase):
    """Assemble a bilinear form into a global ``SparseMatrix``.

    Subclasses select the kernel through ``_tm_form``: ``"diffusion"``
    (``LaplaceElementAssembler``), ``"mass"`` (``MassElementAssembler``) or
    ``"elasticity"`` (``LinearElasticityElementAssembler``)."""

    _tm_form: Optional[str] = None

    def _tm_kind(self) -> Optional[str]:
        """The kernel family of this assembler: the class's ``_tm_form``, or
        for a user subclass the family its ``forward`` is recognised as
        (``recognise_form``), or None for a custom integrand."""
        form = type(self)._tm_form
        if form is not None:
            return form
        rec = recognise_form(self)
        return None if rec is None else rec.form

    def __init__(self, projector, transformation, elements, edges, *args, **kwargs):
        super().__init__()
        if not isinstance(projector, nn.ModuleDict):
            projector = nn.ModuleDict(projector)
        if not isinstance(transformation, nn.ModuleDict):
            transformation = nn.ModuleDict(transformation)
        if not isinstance(elements, BufferDict):
            elements = BufferDict(elements)
        element_types = list(projector.keys())
        self.projector = projector
        self.transformation = transformation
        self.elements = elements
        self.register_buffer("edges", edges)
        self.dimension = element_type2dimension[element_types[0]]
        self.element_types = list(elements.keys())
        self.n_points = next(iter(self.transformation.values())).n_points
        self.__post_init__(*args, **kwargs)

    # -- construction ---------------------------------------------------------
    @classmethod
    def from_mesh(cls, mesh, quadrature_order: int = 2, project: str = "reduce", *args, **kwargs):
        """Build from a mesh (assemble/element_assembler.py:769-878): the CSR
        pattern ``edges`` (int32, unique pairs sorted row-major) and the
        element->CSR slot map are the reference's, computed by the native
        plan builder together with the kernels' reduction plan."""
        assert project in ["reduce", "sparse"]
        points = mesh.points
        elements = _mesh_elements(mesh)
        if len(elements) > 1:
            return cls._from_mixed(mesh, elements, quadrature_order, project, *args, **kwargs)
        etype, conn = _single_type(elements)
        topo = Topology(points, conn, etype, quadrature_order, matrix=True,
                        element_groups=getattr(mesh, "element_groups", None))
        E, B = conn.shape
        if project == "reduce":
            proj = ReduceProjector(indices=topo.slot, from_shape=(E, B, B), to_shape=(topo.nnz,))
        else:
            proj = SparseProjector(from_=torch.arange(E * B * B), to_=topo.slot, from_shape=(E, B, B),
                                   to_shape=(topo.nnz,))
        trans = Transformation(points=points, elements=conn.long(), element_type=etype,
                               quadrature_order=quadrature_order)
        asm = cls({etype: proj}, {etype: trans}, {etype: conn.long()}, topo.edges, *args, **kwargs)
        asm._topology = topo
        return asm.type(mesh.dtype).to(mesh.device)

    @classmethod
    def _from_mixed(cls, mesh, elements, quadrature_order, project, *args, **kwargs):
        """A mesh with several element types (element_assembler.py:811-866):
        one pattern over every type's local pairs, one projector and one
        Transformation per type.  The reference stacks the types' pair
        columns element-major (``torch.stack(..., -1)``), which raises when
        the types have different element counts and, with equal counts,
        hands each type slots of the interleaved sequence; here every type's
        slot map points at the union positions of its own pairs, and the
        assembled matrix is the sum over types."""
        points = mesh.points
        for et in elements:
            element_info(et)
        dims = {element_type2dimension[et] for et in elements}
        if len(dims) != 1:
            raise ValueError(f"element types of different dimensions in one mesh: {list(elements)}")
        topo = MixedTopology(points, {et: c for et, c in elements.items()}, quadrature_order, matrix=True)
        proj, trans = {}, {}
        for et, conn in elements.items():
            E, B = conn.shape
            if project == "reduce":
                proj[et] = ReduceProjector(indices=topo.slot[et], from_shape=(E, B, B), to_shape=(topo.nnz,))
            else:
                proj[et] = SparseProjector(from_=torch.arange(E * B * B), to_=topo.slot[et], from_shape=(E, B, B),
                                           to_shape=(topo.nnz,))
            trans[et] = Transformation(points=points, elements=conn.long(), element_type=et,
                                       quadrature_order=quadrature_order)
        asm = cls(proj, trans, {et: c.long() for et, c in elements.items()}, topo.edges, *args, **kwargs)
        asm._topology = topo
        return asm.type(mesh.dtype).to(mesh.device)

    @classmethod
    def from_assembler(cls, obj, *args, **kwargs):
        """Share the topology of another assembler (element_assembler.py:742-766)."""
        assert isinstance(obj, ElementAssembler), f"obj must be an instance of ElementAssembler, but got {type(obj)}"
        asm = cls(obj.projector, obj.transformation, obj.elements, obj.edges, *args, **kwargs)
        asm._topology = obj._topology
        return asm

    # -- call -----------------------------------------------------------------
    def _prepare(self, points, point_data, element_data, scalar_data):
        assert isinstance(point_data, dict) or point_data is None, \
            f"point_data should be a dict, but got {type(point_data)}"
        et = self.element_types[0]
        trans = self.transformation[et]
        if points is None:
            points = trans.points
        else:
            assert points.shape[1] == trans.dim, \
                f"the dimension of points should be {trans.dim}, but got {points.shape[1]}"
            trans.update_points(points)
        _lib.require_cuda(points, "points")
        self.type(points.dtype).to(points.device)
        E = self.elements[et].shape[0]
        ed = {}
        if element_data:
            for key, value in element_data.items():
                if isinstance(value, dict):
                    value = value[et]
                assert value.shape[0] == E, f"the shape of {key} should be [{E}, ...], but got {tuple(value.shape)}"
                ed[key] = value
        sd = dict(scalar_data or {})
        rec = recognise_form(self)
        if point_data and rec is not None and rec.coef is not None and rec.coef in point_data \
                and rec.coef not in ed:
            ed[_MODULUS_KEY] = self._nodal_modulus(rec, point_data[rec.coef], et, points)
        return et, points, ed, sd

    def _nodal_modulus(self, rec, c_nodes, et, points):
        """The per-element modulus of a form whose coefficient is given per
        node (point_data), interpolated to the quadrature points as the
        reference does (the nodal value times phi at each point): on P1
        elements, whose gradients are constant, the element matrix is the
        unit-modulus one times sum_q w_q m(c(x_q)) / sum_q w_q."""
        if et not in ("triangle", "tetra") or rec.form == "mass":
            raise NotImplementedError("a per-node coefficient is assembled for diffusion and elasticity forms "
                                      "on P1 triangles and tetrahedra")
        tab = element_tables(et, self.transformation[et].quadrature_order)
        dev = points.device
        w = torch.from_numpy(tab["w"]).to(device=dev, dtype=torch.float64)
        phi = torch.from_numpy(tab["phi"]).to(device=dev, dtype=torch.float64)
        c = torch.as_tensor(c_nodes).to(device=dev, dtype=torch.float64).reshape(-1)
        conn = self.elements[et].to(dev).long()
        cq = c[conn] @ phi.T                                          # [E, Q]
        mq = rec.modulus(cq.reshape(-1)).reshape(cq.shape) if (rec.cmap is not None or rec.scale != 1.0) else cq
        return (mq @ w) / w.sum()

    def __call__(self, points: Optional[torch.Tensor] = None, func: Optional[Callable] = None,
                 point_data=None, element_data=None, scalar_data=None, batch_size: int = -1):
        """Assemble into a ``SparseMatrix`` of shape (N, N), or (N*D, N*D) for
        elasticity.  ``batch_size`` (quadrature chunking in the reference)
        does not change results and is accepted and ignored: the kernel
        never materialises the integrand."""
        if func is not None:
            raise NotImplementedError("custom integrands (func=...) are not assembled by tensormesh_gb300")
        form = self._tm_kind()
        if form is None:
            raise NotImplementedError(
                f"{type(self).__name__}.forward is a custom Python weak form; tensormesh_gb300 assembles the "
                f"built-in families (LaplaceElementAssembler / DiffusionElementAssembler, "
                f"MassElementAssembler, LinearElasticityElementAssembler, or a forward that computes "
                f"c * (gradu @ gradv), c * u * v or an isotropic elasticity block)")
        if isinstance(self._topology, MixedTopology):
            return self._call_mixed(points, point_data, element_data, scalar_data)
        et, points, ed, sd = self._prepare(points, point_data, element_data, scalar_data)
        if torch.is_grad_enabled() and (points.requires_grad or any(
                torch.is_tensor(v) and v.requires_grad for v in list(ed.values()) + list(sd.values()))):
            if form == "mass":
                from .adjoint import MassAssembly
                rho = self._tm_coefficients(ed, sd, self.elements[et].shape[0]).get("rho")
                if torch.is_tensor(rho) and rho.numel() != 1:
                    raise NotImplementedError("a per-element coefficient of the mass form is not assembled by "
                                              "tensormesh_gb300 (a scalar one is)")
                rho_t = rho if torch.is_tensor(rho) and rho.requires_grad else None
                values = MassAssembly.apply(points, rho_t, self, dict(sd))
                return self._build_output(values)
            if form == "elasticity":
                c = self._tm_coefficients(ed, sd, self.elements[et].shape[0])
                young, nu = c.get("E"), c.get("nu", 0.3)
                nu_grad = torch.is_tensor(nu) and nu.requires_grad
                if nu_grad and nu.numel() != 1:
                    raise NotImplementedError("a per-element Poisson ratio is not assembled by tensormesh_gb300")
                if points.requires_grad or nu_grad or (torch.is_tensor(young) and young.requires_grad):
                    from .adjoint import ElasticityAssembly
                    if not torch.is_tensor(young):
                        young = torch.tensor(1.0 if young is None else float(young), dtype=torch.float64,
                                             device=points.device)
                    if not torch.is_tensor(nu):
                        nu = torch.tensor(float(nu), dtype=torch.float64)
                    rest = {k: v for k, v in c.items() if k not in ("E", "nu")}
                    values = ElasticityAssembly.apply(young, nu.reshape(()), points, self, rest)
                    return self._build_output(values)
                (values,) = assemble_forms([self], points, ed, sd)
                return self._build_output(values)
            if form != "diffusion":
                raise NotImplementedError(f"gradients of the {form} form are not implemented")
            from .adjoint import DiffusionAssembly
            kap = self._tm_coefficients(ed, sd, self.elements[et].shape[0]).get("kappa")
            if torch.is_tensor(kap) and (kap.dim() > 0 or kap.requires_grad):
                kap = kap.reshape(-1) if kap.numel() > 1 else kap.reshape(())
                values = DiffusionAssembly.apply(points, kap, self, 1.0)
            else:
                values = DiffusionAssembly.apply(points, None, self, 1.0 if kap is None else float(kap))
            return self._build_output(values)
        (values,) = assemble_forms([self], points, ed, sd)
        return self._build_output(values)

    def _call_mixed(self, points, point_data, element_data, scalar_data) -> SparseMatrix:
        et0 = self.element_types[0]
        if points is None:
            points = self.transformation[et0].points
        for et in self.element_types:
            self.transformation[et].update_points(points)
        _lib.require_cuda(points, "points")
        self.type(points.dtype).to(points.device)
        ed = dict(element_data or {})
        sd = dict(scalar_data or {})
        pd = dict(point_data or {})
        leaves = [points] + [v for v in list(ed.values()) + list(sd.values()) + list(pd.values())
                             if torch.is_tensor(v)]
        leaves += [t for v in ed.values() if isinstance(v, dict) for t in v.values() if torch.is_tensor(t)]
        if pd or (torch.is_grad_enabled() and any(t.requires_grad for t in leaves)):
            # each type on its own pattern through the single-type path
            # (per-node coefficients, the adjoint kernels), summed into the
            # union pattern by a differentiable combine
            per_type = _split_element_data(self._topology, ed)
            parts = []
            for et in self._topology.types:
                Kt = self._type_view(et)(points, point_data=pd, element_data=per_type[et], scalar_data=sd)
                H = Kt._block
                parts.append(Kt.values.reshape(-1, H, H) if H > 1 else Kt.values)
            return self._build_output(_CombineParts.apply(self._topology, "matrix", *parts))
        (values,) = assemble_forms([self], points, ed, sd)
        return self._build_output(values)

    def _type_view(self, et: str) -> "ElementAssembler":
        """This assembler restricted to element type ``et`` of a mixed mesh,
        on that type's own pattern (its Topology, slot map and edges), so
        that the single-type path runs on it; kept per type."""
        views = self.__dict__.setdefault("_tm_type_views", {})
        key = (et, self.elements[et].device)
        if key not in views:
            import copy
            topo = self._topology.topos[et]
            sub = copy.copy(self)
            object.__setattr__(sub, "_modules", dict(self._modules))
            object.__setattr__(sub, "_buffers", dict(self._buffers))
            object.__setattr__(sub, "_parameters", dict(self._parameters))
            E, B = self.elements[et].shape
            dev = self.elements[et].device
            sub.projector = nn.ModuleDict({et: ReduceProjector(indices=topo.slot, from_shape=(E, B, B),
                                                               to_shape=(topo.nnz,)).to(dev)})
            sub.transformation = nn.ModuleDict({et: self.transformation[et]})
            sub.elements = BufferDict({et: self.elements[et]})
            sub._buffers["edges"] = topo.edges.to(dev)
            sub.element_types = [et]
            sub._topology = topo
            sub.__dict__.pop("_tm_type_views", None)
            views[key] = sub
        return views[key]

    def _build_output(self, values: torch.Tensor) -> SparseMatrix:
        topo = self._topo(True)
        edges = self.edges
        if values.dim() == 1:
            return SparseMatrix(values, edges[0], edges[1], (self.n_points, self.n_points), _topology=topo,
                                _sorted=True)
        m = SparseMatrix.from_block_coo(values, edges[0], edges[1], (self.n_points, self.n_points),
                                        _topology=topo)
        m._sorted = True
        return m

    # -- form parameters (overridden by the built-ins) ------------------------
    def _tm_coefficients(self, ed, sd, E):
        """Kernel coefficients of a recognised user form: its coefficient
        argument is looked up by name in element_data (per element) or
        scalar_data, as the reference binds forward's arguments."""
        rec = recognise_form(self)
        if rec is None:
            return {}
        if _MODULUS_KEY in ed:                       # from a per-node coefficient, mapped already
            m = ed[_MODULUS_KEY]
            return {"kappa": m} if rec.form == "diffusion" else {"E": m, "nu": rec.nu}
        c = None
        if rec.coef is not None:
            c = ed.get(rec.coef, sd.get(rec.coef))
            if c is None:
                raise KeyError(f"{type(self).__name__}.forward takes {rec.coef!r}: pass it in element_data "
                               f"(one value per element) or scalar_data")
        if rec.form == "mass" and torch.is_tensor(c) and c.dim() > 0 and c.numel() > 1:
            raise NotImplementedError("a per-element coefficient of the mass form is not assembled by "
                                      "tensormesh_gb300 (a scalar one is)")
        m = rec.scale if c is None else rec.modulus(c)
        if rec.form == "diffusion":
            return {"kappa": m}
        if rec.form == "mass":
            return {"rho": m}
        return {"E": m, "nu": rec.nu}

    def forward(self, *args, **kwargs):
        raise NotImplementedError("forward is not implemented")

    def __repr__(self):
        return (f"{type(self).__name__}(element_types={self.element_types}, n_point={self.n_points}, "
                f"n_element={[v.shape[0] for v in self.elements.values()]})")


_FORM_BITS = {"diffusion": _lib.TM_FORM_DIFFUSION, "mass": _lib.TM_FORM_MASS,
              "elasticity": _lib.TM_FORM_ELASTICITY}


def _coef(value, dtype, device, E, name):
    """(pointer tensor or None, scale) for a per-element or scalar coefficient."""
    if value is None:
        return None, 1.0
    if isinstance(value, (int, float)):
        return None, float(value)
    t = torch.as_tensor(value)
    if t.dim() == 0:
        return None, float(t)
    t = t.reshape(-1)
    if t.shape[0] != E:
        raise ValueError(f"{name} must have one value per element ({E}), got {tuple(t.shape)}")
    return t.to(device=device, dtype=dtype).contiguous(), 1.0


def assemble_forms(assemblers, points: Optional[torch.Tensor] = None, element_data=None,
                   scalar_data=None, _events=None, _stats: Optional[torch.Tensor] = None):
    """Assemble several built-in forms over one mesh in one fused launch when
    they can share it (diffusion and mass do), else one launch per form.

    Returns the value tensors ([nnz] per scalar form, [nnz, D, D] for
    elasticity) in the order of ``assemblers``.  ``_events`` (two or three
    ``torch.cuda.Event``) are recorded before and after the element-chunk
    kernel of the first launch and, the third, after that launch's last
    kernel, for timing (any may be None; an event between the two kernels
    makes them run back to back instead of overlapping the second's
    launch); ``_stats`` (a device int32 [1]) counts the chunks whose float64
    P1 locals were recomputed in FP64 arithmetic."""
    first = assemblers[0]
    for a in assemblers[1:]:
        if a._topology is not first._topology:
            raise ValueError("fused assembly needs assemblers that share a topology (from_assembler)")
    leaves = [points] + list((element_data or {}).values()) + list((scalar_data or {}).values())
    leaves += [t for v in (element_data or {}).values() if isinstance(v, dict) for t in v.values()]
    if torch.is_grad_enabled() and any(torch.is_tensor(t) and t.requires_grad for t in leaves):
        # differentiable: each form through its own call (its adjoint kernels)
        out = []
        for a in assemblers:
            m = a(points, element_data=element_data, scalar_data=scalar_data)
            out.append(m.values.reshape(-1, m._block, m._block) if m._block > 1 else m.values)
        return out
    et = first.element_types[0]
    trans = first.transformation[et]
    if points is None:
        points = trans.points
    _lib.require_cuda(points, "points")
    topo = first._topo(True)
    ed = dict(element_data or {})
    sd = dict(scalar_data or {})
    if isinstance(topo, MixedTopology):
        return _assemble_mixed(assemblers, topo, points, ed, sd)
    return _assemble_on(assemblers, topo, points, ed, sd, _events, _stats)


def _split_element_data(topo: "MixedTopology", ed: dict) -> Dict[str, dict]:
    """Per element type, the element data of a mixed mesh: a value given as
    {element_type: tensor} (the reference's per-type form) or as one tensor
    over all elements, the types' elements concatenated in type order."""
    out = {et: {} for et in topo.types}
    total = sum(topo.n_elements.values())
    for key, value in ed.items():
        if isinstance(value, dict):
            for et in topo.types:
                out[et][key] = value[et]
        elif torch.is_tensor(value) and value.dim() > 0:
            if value.shape[0] != total:
                raise ValueError(f"{key} must be a {{element_type: tensor}} dict or have one value per element "
                                 f"of all types ({total}), got {tuple(value.shape)}")
            o = 0
            for et in topo.types:
                n = topo.n_elements[et]
                out[et][key] = value[o:o + n]
                o += n
        else:
            for et in topo.types:
                out[et][key] = value
    return out


def _combine(topo: "MixedTopology", kind: str, parts, dev, dt) -> torch.Tensor:
    """Sum per-type results into the union pattern ("matrix") or onto the
    nodes ("node") with one deterministic gather-sum, types in order."""
    lib = _lib.load()
    width = int(np.prod(parts[0].shape[1:])) if parts[0].dim() > 1 else 1
    x = torch.cat([p.reshape(p.shape[0], width) for p in parts], 0).contiguous()
    n_to = topo.nnz if kind == "matrix" else topo.n_points
    seg, src = topo.segments(dev, kind)
    out = torch.empty(n_to, *parts[0].shape[1:], dtype=dt, device=dev)
    _lib.check(lib.tm_project_reduce(_lib.dtype_code(dt), n_to, width, _lib.ptr(seg), _lib.ptr(src), _lib.ptr(x),
                                     _lib.ptr(out), _lib.stream_handle(dev)), "tm_project_reduce")
    return out


class _CombineParts(torch.autograd.Function):
    """``_combine`` with its gradient: each entry of a part receives the
    gradient of the union position ("matrix") or node ("node") it is summed
    into."""

    @staticmethod
    def forward(ctx, topo, kind, *parts):
        ctx.topo, ctx.kind = topo, kind
        ctx.shapes = [p.shape for p in parts]
        return _combine(topo, kind, [p.detach() for p in parts], parts[0].device, parts[0].dtype)

    @staticmethod
    def backward(ctx, g):
        grads = []
        for et, shape in zip(ctx.topo.types, ctx.shapes):
            if ctx.kind == "matrix":
                grads.append(g[ctx.topo.map_tensor(et, g.device)].reshape(shape))
            else:
                grads.append(g.reshape(shape))
        return (None, None, *grads)


def _assemble_mixed(assemblers, topo: "MixedTopology", points, ed, sd):
    per_type = _split_element_data(topo, ed)
    parts = [_assemble_on(assemblers, topo.topos[et], points, per_type[et], sd, None, None) for et in topo.types]
    return [_combine(topo, "matrix", [p[i] for p in parts], points.device, points.dtype)
            for i in range(len(assemblers))]


def _assemble_on(assemblers, topo: Topology, points, ed, sd, _events, _stats, _coefs=None):
    """The fused launches of ``assemble_forms`` on one element type
    (``_coefs``: the assemblers' kernel coefficients, resolved already)."""
    E = topo.n_elements
    dev, dt = points.device, points.dtype
    pts = points.detach().contiguous()
    if pts.dtype not in (torch.float64, torch.float32):
        raise TypeError(f"points must be float64 or float32, got {pts.dtype}")
    forms = [a._tm_kind() for a in assemblers]
    scalar_group = [i for i, f in enumerate(forms) if f in ("diffusion", "mass")]
    out = [None] * len(assemblers)
    groups = []
    if len(scalar_group) == 2 and forms[scalar_group[0]] != forms[scalar_group[1]]:
        groups.append(scalar_group)
    else:
        groups.extend([[i] for i in scalar_group])
    groups.extend([[i] for i, f in enumerate(forms) if f == "elasticity"])
    lib = _lib.load()
    D = topo.info.dim
    for g in groups:
        bits = 0
        args = _lib.MatrixArgs()
        args.dtype = _lib.dtype_code(dt)
        args.n_points = topo.n_points
        args.points = _lib.ptr(pts)
        args.kappa_scale = args.mass_scale = args.young_scale = 1.0
        args.poisson = 0.3
        keep = [pts]
        block = False
        for i in g:
            a = assemblers[i]
            f = forms[i]
            bits |= _FORM_BITS[f]
            c = _coefs[i] if _coefs is not None else a._tm_coefficients(ed, sd, E)
            if f == "diffusion":
                t, s = _coef(c.get("kappa"), dt, dev, E, "kappa")
                args.kappa, args.kappa_scale = _lib.ptr(t), s
                keep.append(t)
                out[i] = torch.empty(topo.nnz, dtype=dt, device=dev)
                args.out_diffusion = _lib.ptr(out[i])
            elif f == "mass":
                _, s = _coef(c.get("rho"), dt, dev, E, "rho")
                args.mass_scale = s
                out[i] = torch.empty(topo.nnz, dtype=dt, device=dev)
                args.out_mass = _lib.ptr(out[i])
            else:
                block = True
                t, s = _coef(c.get("E"), dt, dev, E, "E")
                args.young, args.young_scale = _lib.ptr(t), s * float(c.get("E_scale", 1.0))
                args.poisson = float(c.get("nu", 0.3))
                keep.append(t)
                out[i] = torch.empty(topo.nnz, D, D, dtype=dt, device=dev)
                args.out_elasticity = _lib.ptr(out[i])
        args.forms = bits
        plan = topo.matrix_plan(dev, block=block, dtype=dt)
        args.plan = plan.struct()
        args.tables = topo.table_struct(dev)
        ws_bytes = lib.tm_matrix_workspace_bytes(C_byref(args))
        ws = torch.empty(max(1, ws_bytes), dtype=torch.uint8, device=dev)
        args.workspace = _lib.ptr(ws)
        if _events is not None:
            ev = lambda e: 0 if e is None else e.cuda_event
            args.event_begin, args.event_end = ev(_events[0]), ev(_events[1])
            if len(_events) > 2:
                args.event_done = ev(_events[2])
            _events = None
        if _stats is not None:
            args.stats = _lib.ptr(_stats)
        _lib.check(lib.tm_assemble_matrix(C_byref(args), _lib.stream_handle(dev)), "tm_assemble_matrix")
    return out


def C_byref(x):
    import ctypes
    return ctypes.byref(x)


# ============================================================================
# Linear forms
# ============================================================================
class NodeAssembler(_AssemblerBase):
    """Assemble a linear form into a nodal vector [N] (or [N*H])."""

    def __init__(self, projector, transformation, elements, *args, **kwargs):
        super().__init__()
        if not isinstance(projector, nn.ModuleDict):
            projector = nn.ModuleDict(projector)
        if not isinstance(transformation, nn.ModuleDict):
            transformation = nn.ModuleDict(transformation)
        if not isinstance(elements, BufferDict):
            elements = BufferDict(elements)
        element_types = list(projector.keys())
        self.projector = projector
        self.transformation = transformation
        self.elements = elements
        self.dimension = element_type2dimension[element_types[0]]
        self.element_types = element_types
        # the reference stores the element count of the first type here
        # (node_assembler.py:130)
        self.n_points = next(iter(elements.values())).shape[0]
        self._compile = False
        self._compile_options = {}
        self.__post_init__(*args, **kwargs)

    @classmethod
    def from_elements(cls, points: torch.Tensor, elements: Dict[str, torch.Tensor], quadrature_order: int = 2,
                      device="cpu", dtype: torch.dtype = torch.float32, project: str = "reduce", *args, **kwargs):
        """node_assembler.py:617-698: the scatter map is conn.flatten()."""
        return cls._build(points, elements, quadrature_order, device, dtype, project, None, *args, **kwargs)

    @classmethod
    def _build(cls, points, elements, quadrature_order, device, dtype, project, element_groups, *args, **kwargs):
        if not isinstance(elements, torch.Tensor) and len(elements) > 1:
            # several element types: one projector (conn.flatten()) and one
            # Transformation per type, the nodal vectors summed over types
            # in type order (node_assembler.py:617-698)
            N = points.shape[0]
            proj, trans = {}, {}
            for et, conn in elements.items():
                element_info(et)
                E, B = conn.shape
                if project == "reduce":
                    proj[et] = ReduceProjector(indices=conn.flatten(), from_shape=(E, B), to_shape=(N,))
                elif project == "sparse":
                    proj[et] = SparseProjector(from_=torch.arange(E * B), to_=conn.flatten(), from_shape=(E, B),
                                               to_shape=(N,))
                else:
                    raise ValueError(f"project should be either 'reduce' or 'sparse', but got {project}")
                trans[et] = Transformation(points, conn, et, quadrature_order)
            asm = cls(proj, trans, dict(elements), *args, **kwargs)
            asm._topology = MixedTopology(points, dict(elements), quadrature_order, matrix=False)
            return asm.type(dtype).to(device)
        etype, conn = _single_type(elements)
        N = points.shape[0]
        E, B = conn.shape
        if project == "reduce":
            proj = ReduceProjector(indices=conn.flatten(), from_shape=(E, B), to_shape=(N,))
        elif project == "sparse":
            proj = SparseProjector(from_=torch.arange(E * B), to_=conn.flatten(), from_shape=(E, B), to_shape=(N,))
        else:
            raise ValueError(f"project should be either 'reduce' or 'sparse', but got {project}")
        trans = Transformation(points, conn, etype, quadrature_order)
        asm = cls({etype: proj}, {etype: trans}, {etype: conn}, *args, **kwargs)
        asm._topology = Topology(points, conn, etype, quadrature_order, matrix=False, element_groups=element_groups)
        return asm.type(dtype).to(device)

    @classmethod
    def from_mesh(cls, mesh, quadrature_order: int = 2, project: str = "reduce", *args, **kwargs):
        elements = _mesh_elements(mesh)
        return cls._build(mesh.points, elements, quadrature_order, mesh.device, mesh.dtype, project,
                          getattr(mesh, "element_groups", None), *args, **kwargs)

    @classmethod
    def from_assembler(cls, obj, *args, **kwargs):
        assert isinstance(obj, NodeAssembler), f"the object {obj} should inherit from NodeAssembler"
        asm = cls(obj.projector, obj.transformation, obj.elements, *args, **kwargs)
        asm._topology = obj._topology
        return asm

    # the reference's compile()/flat_mode switch between its vmap path and a
    # broadcast path; the kernel path is the same either way
    def compile(self, mode: str = "disable", **kwargs):
        self._compile = True
        self._compile_options = {"mode": mode, **kwargs}
        return self

    def flat_mode(self):
        return self.compile(mode="disable")

    def reset_compile(self):
        self._compile = False
        self._compile_options = {}
        return self

    @property
    def is_compiled(self) -> bool:
        return self._compile

    def forward(self, *args, **kwargs):
        raise NotImplementedError("forward is not implemented")

    def __call__(self, points: Optional[torch.Tensor] = None, func: Optional[Callable] = None,
                 point_data=None, scalar_data=None, batch_size: int = 1) -> torch.Tensor:
        if point_data is None:
            point_data = {}
        if scalar_data is None:
            scalar_data = {}
        et = self.element_types[0]
        trans = self.transformation[et]
        if points is None:
            points = trans.points
        else:
            assert points.shape[1] == trans.dim, \
                f"the dimension of the points should be {trans.dim}, but got {points.shape[1]}"
            trans.update_points(points)
        _lib.require_cuda(points, "points")
        self.type(points.dtype).to(points.device)
        for key, value in point_data.items():
            assert value.shape[0] == points.shape[0], \
                f"the shape of {key} should be [n_point, ...], but got {tuple(value.shape)}"
        fn = self.forward if func is None else func
        topo = self._topology
        if isinstance(topo, MixedTopology):
            for et in self.element_types[1:]:
                self.transformation[et].update_points(points)
            parts = [assemble_linear_form(self, fn, points, point_data, scalar_data, topo=topo.topos[et])
                     for et in topo.types]
            width = parts[0].numel() // topo.n_points
            return _CombineParts.apply(topo, "node", *[p.reshape(topo.n_points, width) for p in parts]).reshape(-1)
        return assemble_linear_form(self, fn, points, point_data, scalar_data)


def assemble_linear_form(asm: NodeAssembler, fn: Callable, points: torch.Tensor, point_data, scalar_data,
                         topo: Optional[Topology] = None):
    topo = asm._topo(False) if topo is None else topo
    dev, dt = points.device, points.dtype
    pts = points.detach().contiguous()
    params = list(inspect.signature(fn).parameters)
    if "gradv" in params:
        raise NotImplementedError("linear forms in gradv are not assembled by tensormesh_gb300")
    for p in params:
        if p not in ("v", "x") and p not in point_data and p not in scalar_data and \
                not (p.startswith("grad") and p[4:] in point_data):
            raise ValueError(f"{p} is not supported, please use `v`, `gradv` or more keys provided by "
                             f"point_data or scalar_data")
    source = getattr(asm, "_tm_source", None) if fn == asm.forward else None
    Q = len(element_tables(topo.etype, topo.quadrature_order)["w"])
    E = topo.n_elements
    needs_grad = torch.is_grad_enabled() and (points.requires_grad or any(
        torch.is_tensor(v) and v.requires_grad for v in list(point_data.values()) + list(scalar_data.values())))
    if source is not None and source[0] == "const":
        c = source[1] if torch.is_tensor(source[1]) else torch.as_tensor(source[1], dtype=torch.float64)
        c = c.reshape(-1)
        if needs_grad or (torch.is_grad_enabled() and c.requires_grad):
            from .adjoint import LoadAssembly
            return LoadAssembly.apply(points, c, topo, _lib.TM_SOURCE_CONST, int(c.numel()))
        return _run_vector(topo, pts, _lib.TM_SOURCE_CONST, None, c.tolist(), int(c.numel()))
    if source is not None and source[0] == "nodal" and source[1] in point_data:
        f = point_data[source[1]].to(device=dev, dtype=dt)
        width = 1 if f.dim() == 1 else int(np.prod(f.shape[1:]))
        if needs_grad:
            from .adjoint import LoadAssembly
            return LoadAssembly.apply(points, f, topo, _lib.TM_SOURCE_NODAL, width)
        fv = f.detach().reshape(f.shape[0], width).contiguous()
        return _run_vector(topo, pts, _lib.TM_SOURCE_NODAL, fv, None, width)
    # general source g(x, data) * v: evaluate g at the quadrature points (in
    # torch, so that gradients flow through g to x_q and to its data)
    args = {}
    need_x = "x" in params
    if need_x or any(p.startswith("grad") for p in params):
        if needs_grad and points.requires_grad:
            from .adjoint import QuadPoints
            xq = QuadPoints.apply(points, topo)               # [E, Q, D], differentiable
        else:
            xq = quadrature_points(topo, pts)                 # [E, Q, D]
    phi = torch.from_numpy(element_tables(topo.etype, topo.quadrature_order)["phi"]).to(device=dev, dtype=dt)
    conn = topo.conn32(dev).long()
    for p in params:
        if p == "v":
            args[p] = torch.ones((), dtype=dt, device=dev)
        elif p == "x":
            args[p] = xq
        elif p in point_data:
            v = point_data[p].to(device=dev, dtype=dt)
            args[p] = torch.einsum("eb...,qb->eq...", v[conn], phi)
        elif p in scalar_data:
            args[p] = torch.as_tensor(scalar_data[p], dtype=dt, device=dev)
        else:
            raise NotImplementedError(f"gradient of point data ({p}) in a linear form is not supported")
    g = fn(**args)
    g = torch.as_tensor(g, dtype=dt, device=dev)
    if g.dim() >= 2 and g.shape[0] == E and g.shape[1] == Q:
        trailing = g.shape[2:]
    else:
        trailing = g.shape
        g = g.expand(E, Q, *trailing)
    width = int(np.prod(trailing)) if len(trailing) else 1
    fq = g.reshape(E, Q, width).contiguous()
    if needs_grad or (torch.is_grad_enabled() and fq.requires_grad):    # (tensors captured by the function too)
        from .adjoint import QuadLoadAssembly
        return QuadLoadAssembly.apply(points, fq, topo, width)
    return _run_vector(topo, pts, _lib.TM_SOURCE_QUAD, fq, None, width)


def quadrature_points(topo: Topology, pts: torch.Tensor) -> torch.Tensor:
    lib = _lib.load()
    dev = pts.device
    Q = len(element_tables(topo.etype, topo.quadrature_order)["w"])
    xq = torch.empty(topo.n_elements, Q, topo.info.dim, dtype=pts.dtype, device=dev)
    conn = topo.conn32(dev)
    _lib.check(lib.tm_quadrature_points(_lib.dtype_code(pts.dtype), topo.n_elements, _lib.ptr(conn), _lib.ptr(pts),
                                        topo.table_struct(dev), _lib.ptr(xq), _lib.stream_handle(dev)),
               "tm_quadrature_points")
    return xq


def _run_vector(topo: Topology, pts: torch.Tensor, source: int, values: Optional[torch.Tensor],
                const, width: int) -> torch.Tensor:
    if width > 3:
        raise NotImplementedError("linear forms with more than 3 components per node are not supported")
    lib = _lib.load()
    dev, dt = pts.device, pts.dtype
    plan = topo.node_plan(dev, dtype=dt)
    args = _lib.VectorArgs()
    args.dtype = _lib.dtype_code(dt)
    args.source = source
    args.width = width
    args.n_points = topo.n_points
    args.points = _lib.ptr(pts)
    args.values = _lib.ptr(values)
    if const is not None:
        for k, c in enumerate(const):
            args.constant[k] = float(c)
    out = torch.empty(topo.n_points, width, dtype=dt, device=dev)
    args.out = _lib.ptr(out)
    args.plan = plan.struct()
    args.tables = topo.table_struct(dev)
    ws = torch.empty(max(1, lib.tm_vector_workspace_bytes(C_byref(args))), dtype=torch.uint8, device=dev)
    args.workspace = _lib.ptr(ws)
    _lib.check(lib.tm_assemble_vector(C_byref(args), _lib.stream_handle(dev)), "tm_assemble_vector")
    return out.reshape(-1)
