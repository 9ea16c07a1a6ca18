"""Adjoint gradients dL/dkappa and dL/dx (P1 diffusion + load, Dirichlet
solve) against the reference's autograd gradient (golden fixture), against
central finite differences, and at full size against the oracle's autograd
of the bilinear functional -lambda^T K(kappa, x) u + lambda^T b(x).

Tolerances: 1e-9 relative to the reference's autograd gradient (the solves
are PCG to 1e-14 here, direct there); 1e-8 relative to central differences
(eps = 1e-6, losses from exact dense solves); 1e-10 against the oracle."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import load_golden, rel_fro
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


def _mesh_from_golden(g, dev):
    return tg.Mesh(torch.from_numpy(g["points"]), {"tetra": torch.from_numpy(g["conn"])},
                   {"is_boundary": torch.from_numpy(g["boundary"])}).to(dev)


def test_chain_gradient_matches_reference_autograd(cuda):
    """The reference's own chain: K = asm(x, kappa), b = load(x), condense,
    solve, loss.backward() -- through DiffusionAssembly / LoadAssembly /
    SparseSolve."""
    g = load_golden("adjoint")
    mesh = _mesh_from_golden(g, cuda)
    asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    src = tg.LoadNodeAssembler.from_mesh(mesh)
    pts = mesh.points.clone().requires_grad_(True)
    kappa = torch.from_numpy(g["kappa"]).to(cuda).requires_grad_(True)
    u_t = torch.from_numpy(g["u_target"]).to(cuda)
    mask = mesh.boundary_mask
    K = asm(pts, element_data={"kappa": kappa})
    b = src(pts, point_data={"f": torch.ones(mesh.n_points, dtype=torch.float64, device=cuda)})
    Kc, bc = tg.Condenser(mask)(K, b)
    u = Kc.solve(bc, rtol=1e-14)
    loss = ((u - u_t[~mask]) ** 2).sum()
    loss.backward()
    assert abs(loss.item() - float(g["loss"])) <= 1e-12 * float(g["loss"])
    assert rel_fro(kappa.grad, g["grad_kappa"]) <= 1e-9
    assert rel_fro(pts.grad, g["grad_points"]) <= 1e-9


def test_fused_adjoint_matches_reference_autograd(cuda):
    g = load_golden("adjoint")
    mesh = _mesh_from_golden(g, cuda)
    asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    src = tg.LoadNodeAssembler.from_mesh(mesh)
    cond = tg.Condenser(mesh.boundary_mask)
    pts = mesh.points.clone().requires_grad_(True)
    kappa = torch.from_numpy(g["kappa"]).to(cuda).requires_grad_(True)
    u_t = torch.from_numpy(g["u_target"]).to(cuda)
    ones = torch.ones(mesh.n_points, dtype=torch.float64, device=cuda)
    u = tg.solve_diffusion(asm, src, cond, pts, kappa, f=ones, rtol=1e-14)
    loss = ((u - u_t) ** 2)[~mesh.boundary_mask].sum()
    loss.backward()
    assert rel_fro(kappa.grad, g["grad_kappa"]) <= 1e-9
    assert rel_fro(pts.grad, g["grad_points"]) <= 1e-9


def _dense_loss(mesh, pts, kappa, u_t):
    """Loss with the kernels' K and b and an exact dense solve (for FD)."""
    asm = tg.LaplaceElementAssembler.from_mesh(tg.Mesh(pts, mesh.cells, mesh.point_data))
    src = tg.const_node_assembler(1.0).from_mesh(tg.Mesh(pts, mesh.cells, mesh.point_data))
    with torch.no_grad():
        K = asm(pts, element_data={"kappa": kappa})
        b = src(pts)
        mask = mesh.boundary_mask
        Kd = K.to_dense()[~mask][:, ~mask]
        u = torch.linalg.solve(Kd, b[~mask])
        return float(((u - u_t[~mask]) ** 2).sum())


def test_adjoint_against_central_differences(cuda):
    mesh = tg.gen_unit_cube(6, jitter=0.15, seed=41).to(cuda)
    rng = np.random.default_rng(42)
    kappa0 = torch.from_numpy(rng.lognormal(0.0, 0.5, mesh.n_elements)).to(cuda)
    u_t = torch.from_numpy(rng.uniform(0.0, 0.05, mesh.n_points)).to(cuda)
    asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    src = tg.const_node_assembler(1.0).from_mesh(mesh)
    cond = tg.Condenser(mesh.boundary_mask)
    pts = mesh.points.clone().requires_grad_(True)
    kappa = kappa0.clone().requires_grad_(True)
    u = tg.solve_diffusion(asm, src, cond, pts, kappa, rtol=1e-14)
    loss = ((u - u_t) ** 2)[~mesh.boundary_mask].sum()
    loss.backward()
    eps = 1e-6
    gk = kappa.grad
    gx = pts.grad
    els = rng.choice(mesh.n_elements, 32, replace=False)
    for e in els:
        kp, km = kappa0.clone(), kappa0.clone()
        kp[e] *= 1 + eps
        km[e] *= 1 - eps
        fd = (_dense_loss(mesh, mesh.points, kp, u_t) - _dense_loss(mesh, mesh.points, km, u_t)) / (2 * eps * kappa0[e])
        assert abs(fd - float(gk[e])) <= 1e-8 * float(gk.abs().max()) + 1e-6 * abs(float(gk[e])), (e, fd, float(gk[e]))
    interior = torch.nonzero(~mesh.boundary_mask).reshape(-1).cpu().numpy()
    nodes = rng.choice(interior, 32, replace=False)
    for n in nodes:
        d = int(rng.integers(0, 3))
        pp, pm = mesh.points.clone(), mesh.points.clone()
        pp[n, d] += eps
        pm[n, d] -= eps
        fd = (_dense_loss(mesh, pp, kappa0, u_t) - _dense_loss(mesh, pm, kappa0, u_t)) / (2 * eps)
        assert abs(fd - float(gx[n, d])) <= 1e-8 * float(gx.abs().max()) + 1e-6 * abs(float(gx[n, d])), \
            (n, d, fd, float(gx[n, d]))


def test_adjoint_kernel_full_size_inverse_diffusion_48(cuda):
    """663,552 tets: the fused adjoint against the oracle's autograd of
    -lambda^T K(kappa, x) u + lambda^T b(x) with the same u and lambda."""
    from tensormesh_gb300 import workloads as W
    wl = W.inverse_diffusion_tet(48)
    mesh = wl.mesh.to(cuda)
    asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    src = tg.const_node_assembler(1.0).from_mesh(mesh)
    cond = tg.Condenser(mesh.boundary_mask)
    kappa_t = wl.data["kappa_true"].to(cuda)
    with torch.no_grad():
        u_target = tg.solve_diffusion(asm, src, cond, mesh.points, kappa_t, rtol=1e-12)
    pts = mesh.points.clone().requires_grad_(True)
    kappa = torch.ones(mesh.n_elements, dtype=torch.float64, device=cuda, requires_grad=True)
    u = tg.solve_diffusion(asm, src, cond, pts, kappa, rtol=1e-12)
    loss = ((u - u_target) ** 2).sum()
    loss.backward()
    # the adjoint the backward used: K lambda = 2 (u - u_target) on the free nodes
    with torch.no_grad():
        K = asm(mesh.points, element_data={"kappa": kappa.detach()})
        b = src(mesh.points)
        Ki, _ = cond(K, b)
        lam = cond.prolong(tg.pcg_solve(Ki, cond.restrict(2 * (u - u_target)), rtol=1e-12))
    P = wl.mesh.points.clone().requires_grad_(True)
    kap = torch.ones(mesh.n_elements, dtype=torch.float64, requires_grad=True)
    conn = wl.mesh.elements()
    _, _, Ko = O.assemble_matrix(P, conn, wl.mesh.n_points,
                                 lambda p, c, kappa: O.element_locals_diffusion(p, c, "tetra", kappa, 2), kappa=kap)
    bo = O.assemble_load(P, conn, "tetra", wl.mesh.n_points, const=1.0)
    edges, _ = O.element_pattern(conn, wl.mesh.n_points)
    lc, uc = lam.cpu(), u.detach().cpu()
    J = -(lc[edges[0].long()] * Ko * uc[edges[1].long()]).sum() + (lc * bo).sum()
    J.backward()
    assert rel_fro(kappa.grad, kap.grad) <= 1e-10
    assert rel_fro(pts.grad, P.grad) <= 1e-10
