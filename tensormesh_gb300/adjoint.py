"""Differentiation of the assembly path with hand-written adjoint kernels.

The reference differentiates by running torch autograd through its
assembly graph and a solver adjoint (sparse/solve/torch_sla_solve.py:90-137,
docs/source/user_guide/differentiability.rst:34-56).  Here:

* ``DiffusionAssembly`` -- the values of a P1 diffusion matrix as a function
  of node coordinates and per-element kappa; its backward runs the
  ``tm_adjoint_p1`` kernel on dL/dvalues (CSR weights through the slot map).
* ``MassAssembly`` -- the values of a P1 mass matrix as a function of node
  coordinates and its scalar density; its backward runs ``tm_adjoint_p1``
  in its mass mode (d|det J| / dJ = |det J| J^-T per element).
* ``ElasticityAssembly`` -- the values of an isotropic elasticity matrix as
  a function of its modulus (``tm_coef_grad``: dL/dE_e is the
  contraction of dL/dvalues with the element's blocks at unit modulus).
* ``LoadAssembly`` -- a load vector (any element type) as a function of
  node coordinates and of its constant or nodal source.
* ``SparseSolve`` -- x = A^-1 b with Jacobi-PCG; backward solves A^T lambda =
  dL/dx (A symmetric) and returns dL/dvalues = -lambda_row x_col, dL/db = lambda.
* ``solve_diffusion`` -- the fused form for losses through a Dirichlet
  diffusion solve: forward assembles, condenses and solves; backward solves
  the adjoint system once and runs ``tm_adjoint_p1`` with the weights
  -lambda_a u_b formed per element, so dL/dK is never materialised and the
  geometry is recomputed instead of stored.
"""
import ctypes as C
from typing import Optional

import torch

from . import _lib
from .element import element_tables


def _adjoint_call(topo, points, kappa, kappa_scale, k_mode, weights=None, slot=None, u=None, lam=None,
                  load_source=_lib.TM_ADJ_LOAD_NONE, load_const=0.0, load_values=None,
                  want_kappa=True, want_points=True, poisson=0.3):
    """``tm_adjoint_p1`` on P1 elements, ``tm_adjoint_general`` (per
    quadrature point; diffusion, mass and elasticity weights only) on the
    others and for elasticity on every element type."""
    lib = _lib.load()
    dev = points.device
    pts = points.detach().to(torch.float64).contiguous()
    E = topo.n_elements
    plan = topo.node_plan(dev)          # static chunk size (the tuner times assembly calls only)
    a = _lib.AdjointArgs()
    a.dtype = _lib.TM_F64
    a.k_mode = k_mode
    a.load_source = load_source
    a.n_points = topo.n_points
    a.points = _lib.ptr(pts)
    kap = None if kappa is None else kappa.detach().to(torch.float64).contiguous()
    a.kappa = _lib.ptr(kap)
    a.kappa_scale = float(kappa_scale)
    wts = None if weights is None else weights.detach().to(torch.float64).contiguous()
    a.weights = _lib.ptr(wts)
    a.slot_map = _lib.ptr(slot)
    uu = None if u is None else u.detach().to(torch.float64).contiguous()
    ll = None if lam is None else lam.detach().to(torch.float64).contiguous()
    a.u, a.lam = _lib.ptr(uu), _lib.ptr(ll)
    a.load_const = float(load_const)
    lv = None if load_values is None else load_values.detach().to(torch.float64).contiguous()
    a.load_values = _lib.ptr(lv)
    a.poisson = float(poisson)
    gk = torch.empty(E, dtype=torch.float64, device=dev) if want_kappa else None
    gp = torch.empty(topo.n_points, topo.info.dim, dtype=torch.float64, device=dev) if want_points else None
    a.grad_kappa, a.grad_points = _lib.ptr(gk), _lib.ptr(gp)
    a.plan = plan.struct()
    a.tables = topo.table_struct(dev)
    ws = torch.empty(max(1, lib.tm_adjoint_workspace_bytes(C.byref(a))), dtype=torch.uint8, device=dev)
    a.workspace = _lib.ptr(ws)
    if topo.etype in ("triangle", "tetra") and k_mode != _lib.TM_ADJ_E_CSR and load_source != _lib.TM_ADJ_LOAD_QUAD:
        _lib.check(lib.tm_adjoint_p1(C.byref(a), _lib.stream_handle(dev)), "tm_adjoint_p1")
    else:
        _lib.check(lib.tm_adjoint_general(C.byref(a), _lib.stream_handle(dev)), "tm_adjoint_general")
    return gk, gp


def _require_p1(topo):
    if topo.etype not in ("triangle", "tetra"):
        raise NotImplementedError("gradients are implemented for P1 triangles and tetrahedra")


class DiffusionAssembly(torch.autograd.Function):
    """values = K(points, kappa) of a LaplaceElementAssembler (float64, P1)."""

    @staticmethod
    def forward(ctx, points, kappa, asm, kappa_scale):
        from .assemble import _assemble_on
        # the kernel's coefficient as given (already the form's modulus)
        c = {"kappa": kappa_scale if kappa is None else kappa.detach()}
        (values,) = _assemble_on([asm], asm._topo(True), points.detach(), {}, {}, None, None, _coefs=[c])
        ctx.asm = asm
        ctx.kappa_scale = kappa_scale if kappa is not None else kappa_scale
        ctx.save_for_backward(points, kappa if kappa is not None else torch.empty(0))
        ctx.has_kappa = kappa is not None
        return values

    @staticmethod
    def backward(ctx, gvals):
        points, kappa = ctx.saved_tensors
        asm = ctx.asm
        topo = asm._topology
        et = asm.element_types[0]
        slot = asm.projector[et].indices.to(points.device)
        want_k = ctx.has_kappa and ctx.needs_input_grad[1]
        scalar_k = ctx.has_kappa and kappa.dim() == 0
        if scalar_k or (topo.etype not in ("triangle", "tetra") and not ctx.needs_input_grad[0]):
            # the coefficient alone (any element type): the contraction of
            # dL/dvalues with the unit-coefficient element matrices
            if ctx.needs_input_grad[0]:
                raise NotImplementedError("gradients with respect to both the node coordinates and a "
                                          "scalar kappa are not implemented")
            gk = None
            if want_k:
                g = coef_grad(topo, points, gvals, slot, _lib.TM_FORM_DIFFUSION, 1.0)
                gk = g.sum().reshape(()) if scalar_k else g
            return None, (gk.to(kappa.dtype) if gk is not None else None), None, None
        kap = kappa if ctx.has_kappa else None
        gk, gp = _adjoint_call(topo, points, kap, ctx.kappa_scale, _lib.TM_ADJ_K_CSR, weights=gvals, slot=slot,
                               want_kappa=want_k, want_points=ctx.needs_input_grad[0])
        return (gp.to(points.dtype) if gp is not None else None,
                gk.to(kappa.dtype) if gk is not None else None, None, None)


class MassAssembly(torch.autograd.Function):
    """values = M(points, rho) of a mass form (float64, P1; rho a scalar)."""

    @staticmethod
    def forward(ctx, points, rho, asm, sd):
        from .assemble import assemble_forms
        sdd = {k: (v.detach() if torch.is_tensor(v) else v) for k, v in sd.items()}
        (values,) = assemble_forms([asm], points.detach(), {}, sdd)
        ctx.asm = asm
        r = asm._tm_coefficients({}, sdd, asm._topology.n_elements).get("rho")
        ctx.rho = 1.0 if r is None else float(r)            # the kernel's mass scale
        ctx.save_for_backward(points, values)
        ctx.has_rho = rho is not None
        return values

    @staticmethod
    def backward(ctx, gvals):
        points, values = ctx.saved_tensors
        asm = ctx.asm
        topo = asm._topology
        et = asm.element_types[0]
        slot = asm.projector[et].indices.to(points.device)
        gp = None
        if ctx.needs_input_grad[0]:
            _, gp = _adjoint_call(topo, points, None, ctx.rho, _lib.TM_ADJ_M_CSR, weights=gvals, slot=slot,
                                  want_kappa=False, want_points=True)
            gp = gp.to(points.dtype)
        grho = None
        if ctx.has_rho and ctx.needs_input_grad[1]:
            # M is linear in rho: dL/drho = sum_i gvals_i M_i / rho (rho != 0), else from rho = 1
            if ctx.rho != 0.0:
                grho = (gvals * values).sum() / ctx.rho
            else:
                (m1,) = _mass_unit(asm, points)
                grho = (gvals * m1).sum()
        return gp, grho, None, None


def _mass_unit(asm, points):
    """The mass values at unit density (the kernel's mass scale 1)."""
    from .assemble import assemble_forms
    from .builtin import MassElementAssembler
    unit = MassElementAssembler.from_assembler(asm) if not isinstance(asm, MassElementAssembler) else asm
    return assemble_forms([unit], points.detach(), {}, {"rho": 1.0})


def coef_grad(topo, points, gvals, slot, form, scale, poisson=0.3, lame_parts=False):
    """dL/dc_e = scale sum_ab W[slot(e,a,b)] : K_e[a][b](c = 1), element
    order (``tm_coef_grad``; form TM_FORM_DIFFUSION or TM_FORM_ELASTICITY).
    ``lame_parts`` (elasticity): [2E], the contractions with the unit-lam and
    the unit-mu parts of K_e apart."""
    lib = _lib.load()
    dev = points.device
    pts = points.detach().to(torch.float64).contiguous()
    w = gvals.detach().to(torch.float64).contiguous()
    plan = topo.node_plan(dev)
    a = _lib.CoefGradArgs()
    a.form = form
    a.n_points = topo.n_points
    a.points, a.weights, a.slot_map = _lib.ptr(pts), _lib.ptr(w), _lib.ptr(slot)
    a.scale, a.poisson = float(scale), float(poisson)
    a.flags = _lib.TM_COEF_GRAD_LAME_PARTS if lame_parts else 0
    g = torch.empty((2 if lame_parts else 1) * topo.n_elements, dtype=torch.float64, device=dev)
    a.grad = _lib.ptr(g)
    a.tables = topo.table_struct(dev)
    a.plan = plan.struct()
    _lib.check(lib.tm_coef_grad(C.byref(a), _lib.stream_handle(dev)), "tm_coef_grad")
    return g


class ElasticityAssembly(torch.autograd.Function):
    """values = K(E, nu, points) of an isotropic elasticity form (float64,
    any element type) as a function of its modulus E (per element or a
    scalar tensor), its Poisson ratio nu (a scalar tensor) and the node
    coordinates (``coefs``: the form's other kernel coefficients, E_scale);
    the backward runs ``tm_coef_grad`` (dL/dE, and for dL/dnu its unit-lam
    and unit-mu parts apart: K = E (lam'(nu) K_lam + mu'(nu) K_mu)) and
    ``tm_adjoint_general`` in elasticity mode (dL/dpoints) on dL/dvalues."""

    @staticmethod
    def forward(ctx, young, nu, points, asm, coefs):
        from .assemble import _assemble_on
        c = dict(coefs, E=young.detach(), nu=float(nu))
        (values,) = _assemble_on([asm], asm._topo(True), points.detach(), {}, {}, None, None, _coefs=[c])
        ctx.asm, ctx.nu, ctx.escale = asm, float(nu), float(c.get("E_scale", 1.0))
        ctx.save_for_backward(points, young)
        return values

    @staticmethod
    def backward(ctx, gvals):
        points, young = ctx.saved_tensors
        asm = ctx.asm
        et = asm.element_types[0]
        slot = asm.projector[et].indices.to(points.device)
        topo = asm._topology
        per_element = young.dim() > 0 and young.numel() > 1
        gy = gnu = gp = None
        if ctx.needs_input_grad[1]:
            nu = ctx.nu
            parts = coef_grad(topo, points, gvals, slot, _lib.TM_FORM_ELASTICITY, ctx.escale, nu, lame_parts=True)
            pl, pm = parts[:topo.n_elements], parts[topo.n_elements:]
            lam, mu = nu / ((1.0 + nu) * (1.0 - 2.0 * nu)), 1.0 / (2.0 * (1.0 + nu))
            dlam = (1.0 + 2.0 * nu * nu) / ((1.0 + nu) ** 2 * (1.0 - 2.0 * nu) ** 2)
            dmu = -1.0 / (2.0 * (1.0 + nu) ** 2)
            ey = young.detach().reshape(-1).to(parts.device, torch.float64)
            gnu = (ey * (dlam * pl + dmu * pm)).sum().reshape(()).to(torch.float64)
            g = lam * pl + mu * pm
        elif ctx.needs_input_grad[0]:
            g = coef_grad(topo, points, gvals, slot, _lib.TM_FORM_ELASTICITY, ctx.escale, ctx.nu)
        if ctx.needs_input_grad[0]:
            gy = (g if per_element else g.sum().reshape(young.shape)).to(young.dtype)
        if ctx.needs_input_grad[2]:
            ey = young.detach().reshape(-1) if per_element else None
            scale = ctx.escale * (1.0 if per_element else float(young.detach().reshape(())))
            _, gp = _adjoint_call(topo, points, ey, scale, _lib.TM_ADJ_E_CSR, weights=gvals, slot=slot,
                                  want_kappa=False, want_points=True, poisson=ctx.nu)
            gp = gp.to(points.dtype)
        return gy, gnu, gp, None, None


class LoadAssembly(torch.autograd.Function):
    """b(points, s) = sum_q w_q |det J_q| phi_a(q) f(q) for a constant
    (``src`` [W]) or nodal (``src`` [N, W]) source, any element type.
    dL/dpoints runs the load term of ``tm_adjoint_p1`` / ``tm_adjoint_general``
    (one call per component for a nodal source; for a constant one the
    components fold into one weight lam . c); dL/dsrc is linear: the load
    vector of the nodal source lam (the mass matrix applied to lam), or
    lam_k . b(c = 1) per constant component."""

    @staticmethod
    def forward(ctx, points, src, topo, source, width):
        from .assemble import _run_vector
        ctx.topo, ctx.source, ctx.width = topo, source, width
        s = src.detach()
        ctx.save_for_backward(points, s)
        pts = points.detach().contiguous()
        if source == _lib.TM_SOURCE_CONST:
            return _run_vector(topo, pts, source, None, s.reshape(-1).tolist(), width)
        vals = s.reshape(topo.n_points, width).to(device=pts.device, dtype=pts.dtype).contiguous()
        return _run_vector(topo, pts, source, vals, None, width)

    @staticmethod
    def backward(ctx, gb):
        from .assemble import _run_vector
        points, s = ctx.saved_tensors
        topo, W, N = ctx.topo, ctx.width, ctx.topo.n_points
        pts = points.detach().contiguous()
        lam = gb.detach().reshape(N, W)
        gp = gs = None
        if ctx.needs_input_grad[0]:
            if ctx.source == _lib.TM_SOURCE_CONST:
                c = s.reshape(W).to(device=lam.device, dtype=torch.float64)
                _, gp = _adjoint_call(topo, points, None, 1.0, _lib.TM_ADJ_K_NONE,
                                      lam=lam.to(torch.float64) @ c, load_source=_lib.TM_ADJ_LOAD_CONST,
                                      load_const=1.0, want_kappa=False)
            else:
                f = s.reshape(N, W).to(device=lam.device, dtype=torch.float64)
                for k in range(W):
                    _, g = _adjoint_call(topo, points, None, 1.0, _lib.TM_ADJ_K_NONE, lam=lam[:, k],
                                         load_source=_lib.TM_ADJ_LOAD_NODAL, load_values=f[:, k],
                                         want_kappa=False)
                    gp = g if gp is None else gp + g
            gp = gp.to(points.dtype)
        if ctx.needs_input_grad[1]:
            lt = lam.to(pts.dtype).contiguous()
            if ctx.source == _lib.TM_SOURCE_CONST:
                b1 = _run_vector(topo, pts, ctx.source, None, [1.0] * W, W).reshape(N, W)
                gs = (lt * b1).sum(0)
            else:
                gs = _run_vector(topo, pts, _lib.TM_SOURCE_NODAL, lt, None, W)
            gs = gs.reshape(s.shape).to(device=s.device, dtype=s.dtype)
        return gp, gs, None, None, None


def _jxw(topo, points) -> torch.Tensor:
    """w_q |det J_q| per (element, quadrature point), element order."""
    lib = _lib.load()
    dev = points.device
    pts = points.detach().to(torch.float64).contiguous()
    conn = topo.conn32(dev)
    tb = topo.table_struct(dev)
    E, Q, B, D = topo.n_elements, tb.n_quad, topo.info.n_basis, topo.info.dim
    grad = torch.empty(E, Q, B, D, dtype=torch.float64, device=dev)
    jxw = torch.empty(E, Q, dtype=torch.float64, device=dev)
    _lib.check(lib.tm_shape_grad_jxw(E, _lib.ptr(conn), _lib.ptr(pts), tb, _lib.ptr(grad), _lib.ptr(jxw),
                                     _lib.stream_handle(dev)), "tm_shape_grad_jxw")
    return jxw


def _phi(topo, device) -> torch.Tensor:
    from .element import element_tables
    return torch.from_numpy(element_tables(topo.etype, topo.quadrature_order)["phi"]).to(device=device,
                                                                                     dtype=torch.float64)


class QuadLoadAssembly(torch.autograd.Function):
    """b(points, fq)_a = sum_e sum_q w_q |det J_q| phi_a(q) fq[e, q, k]: a
    source given at the quadrature points (``func`` sources, evaluated in
    torch on the quadrature points).  dL/dfq = w_q |det J_q| lam(x_q)
    (lam interpolated with phi); dL/dpoints through |det J_q| by the
    quadrature-point load term of ``tm_adjoint_general``, per component."""

    @staticmethod
    def forward(ctx, points, fq, topo, width):
        from .assemble import _run_vector
        ctx.topo, ctx.width = topo, width
        f = fq.detach().contiguous()
        ctx.save_for_backward(points, f)
        return _run_vector(topo, points.detach().contiguous(), _lib.TM_SOURCE_QUAD, f, None, width)

    @staticmethod
    def backward(ctx, gb):
        points, f = ctx.saved_tensors
        topo, W = ctx.topo, ctx.width
        dev = gb.device
        lam = gb.detach().to(torch.float64).reshape(topo.n_points, W)
        gp = gf = None
        if ctx.needs_input_grad[1]:
            conn = topo.conn32(dev).long()
            lamq = torch.einsum("ebk,qb->eqk", lam[conn], _phi(topo, dev))
            gf = (_jxw(topo, points)[..., None] * lamq).reshape(f.shape).to(f.dtype)
        if ctx.needs_input_grad[0]:
            E = topo.n_elements
            fk = f.to(torch.float64).reshape(E, -1, W)
            for k in range(W):
                _, g = _adjoint_call(topo, points, None, 1.0, _lib.TM_ADJ_K_NONE, lam=lam[:, k],
                                     load_source=_lib.TM_ADJ_LOAD_QUAD, load_values=fk[:, :, k].reshape(-1),
                                     want_kappa=False)
                gp = g if gp is None else gp + g
            gp = gp.to(points.dtype)
        return gp, gf, None, None


class QuadPoints(torch.autograd.Function):
    """x_q = sum_b phi_b(q) x_b per (element, quadrature point)
    (``tm_quadrature_points``); dL/dx_b = sum_(e,q) phi_b(q) dL/dx_q, formed
    as the load vector of the quadrature values dL/dx_q / (w_q |det J_q|)."""

    @staticmethod
    def forward(ctx, points, topo):
        from .assemble import quadrature_points
        ctx.topo = topo
        ctx.save_for_backward(points)
        return quadrature_points(topo, points.detach().contiguous())

    @staticmethod
    def backward(ctx, gx):
        from .assemble import _run_vector
        (points,) = ctx.saved_tensors
        topo = ctx.topo
        D = gx.shape[-1]
        jxw = _jxw(topo, points)
        vals = (gx.detach().to(torch.float64) / jxw[..., None]).contiguous()
        gp = _run_vector(topo, points.detach().to(torch.float64).contiguous(), _lib.TM_SOURCE_QUAD, vals, None, D)
        return gp.reshape(points.shape).to(points.dtype), None


class SparseSolve(torch.autograd.Function):
    """x = A^-1 b for a SparseMatrix A: Jacobi-PCG (``method="cg"``, A
    symmetric positive definite) or Jacobi-BiCGSTAB (``"bicgstab"``).  The
    backward solves A^T lam = dL/dx and returns dL/db = lam and dL/dA_ij =
    -lam_i x_j (the reference's SparseSolveTorch.backward,
    sparse/solve/torch_solve.py:262-270)."""

    @staticmethod
    def forward(ctx, values, b, A, kwargs):
        from .solve import bicgstab_solve, pcg_solve
        kw = dict(kwargs)
        method = kw.pop("method", "cg")
        info_out = kw.pop("_info_out", None)       # a list that receives the forward solve's SolveInfo
        kw.pop("return_info", None)
        solver = pcg_solve if method == "cg" else bicgstab_solve
        x, info = solver(A.with_values(values.detach()), b.detach(), return_info=True, **kw)
        if info_out is not None:
            info_out.append(info)
        kw.pop("x0", None)
        ctx.A, ctx.kwargs, ctx.solver, ctx.method = A, kw, solver, method
        ctx.save_for_backward(values, x)
        return x

    @staticmethod
    def backward(ctx, gx):
        values, x = ctx.saved_tensors
        A = ctx.A.with_values(values.detach())
        At = A if ctx.method == "cg" else A.transpose()
        lam = ctx.solver(At, gx.detach(), **ctx.kwargs)
        gvals = None
        if ctx.needs_input_grad[0]:
            gvals = -lam[A.row_indices] * x[A.col_indices]
        return gvals, lam, None, None


class _DiffusionSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, points, kappa, asm, load, condenser, f, rtol):
        from .assemble import assemble_forms
        from .solve import pcg_solve
        topo = asm._topology
        ed = {"kappa": kappa.detach()}
        (values,) = assemble_forms([asm], points.detach(), ed)
        K = asm._build_output(values)
        if f is None:
            b = load(points.detach())
        else:
            b = load(points.detach(), point_data={"f": f})
        Ki, bi = condenser(K, b)
        ui = pcg_solve(Ki, bi, rtol=rtol)
        u = condenser.recover(ui)
        ctx.asm, ctx.load, ctx.cond, ctx.Ki, ctx.rtol = asm, load, condenser, Ki, rtol
        ctx.save_for_backward(points, kappa, u, f if f is not None else torch.empty(0))
        ctx.has_f = f is not None
        return u

    @staticmethod
    def backward(ctx, gu):
        from .solve import pcg_solve
        points, kappa, u, f = ctx.saved_tensors
        topo = ctx.asm._topology
        _require_p1(topo)
        cond = ctx.cond
        lam_i = pcg_solve(ctx.Ki, cond.restrict(gu.detach().to(torch.float64)), rtol=ctx.rtol)
        lam = cond.prolong(lam_i)
        source = getattr(ctx.load, "_tm_source", None)
        if ctx.has_f:
            load, lconst, lvals = _lib.TM_ADJ_LOAD_NODAL, 0.0, f
        elif source is not None and source[0] == "const":
            load, lconst, lvals = _lib.TM_ADJ_LOAD_CONST, float(torch.as_tensor(source[1])), None
        else:
            raise NotImplementedError("solve_diffusion: the load must be a constant or a nodal source")
        gk, gp = _adjoint_call(topo, points, kappa, 1.0, _lib.TM_ADJ_K_OUTER, u=u, lam=lam, load_source=load,
                               load_const=lconst, load_values=lvals,
                               want_kappa=ctx.needs_input_grad[1], want_points=ctx.needs_input_grad[0])
        return (gp.to(points.dtype) if gp is not None else None, gk.to(kappa.dtype) if gk is not None else None,
                None, None, None, None, None)


def solve_diffusion(asm, load, condenser, points: torch.Tensor, kappa: torch.Tensor,
                    f: Optional[torch.Tensor] = None, rtol: float = 1e-12) -> torch.Tensor:
    """u(points, kappa) solving K(kappa, points) u = b(points) with the
    Dirichlet data of ``condenser``; differentiable in ``points`` and
    ``kappa`` through the fused adjoint (one adjoint PCG solve and one
    element pass per backward)."""
    return _DiffusionSolve.apply(points, kappa, asm, load, condenser, f, rtol)
