"""Adjoint gradients dL/dkappa and dL/dx (P1 diffusion + load, Dirichlet
solve) against the reference's autograd gradient (golden fixture), against
central finite differences, and at full size against the oracle's autograd
of the bilinear functional -lambda^T K(kappa, x) u + lambda^T b(x).

Tolerances: 1e-9 relative to the reference's autograd gradient (the solves
are PCG to 1e-14 here, direct there); 1e-8 relative to central differences
(eps = 1e-6, losses from extended-precision dense solves); 1e-10 against
the oracle."""
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


def _solve_spd_extended(A, b):
    """Gaussian elimination without pivoting (A is SPD) in numpy longdouble."""
    A = A.copy()
    b = b.copy()
    n = A.shape[0]
    for k in range(n - 1):
        f = A[k + 1:, k] / A[k, k]
        A[k + 1:, k:] -= f[:, None] * A[k, k:][None, :]
        b[k + 1:] -= f * b[k]
    x = np.zeros(n, dtype=A.dtype)
    for k in range(n - 1, -1, -1):
        x[k] = (b[k] - A[k, k + 1:] @ x[k + 1:]) / A[k, k]
    return x


def _p1_tet_system_extended(pts, conn, kappa, n):
    """Dense K(kappa) and load b (f = 1) of P1 tets in numpy longdouble, with
    the same quadrature nodes and weights (order 2) as the float64 path:
    K_e = kappa_e sum_q w_q |det A| G G^T, b_a = sum_q w_q |det A| phi_a(xi_q),
    G the barycentric gradients (columns of A^-1, A the edge matrix)."""
    L = np.longdouble
    w, xi = (t.numpy().astype(L) for t in O.quadrature("tetra", 2))
    phi = np.concatenate([1 - xi.sum(1, keepdims=True), xi], 1)          # [Q, 4]
    X = pts.astype(L)[conn]                                              # [E, 4, 3]
    A = X[:, 1:] - X[:, :1]                                              # rows x_i - x_0
    c0 = np.cross(A[:, 1], A[:, 2])
    c1 = np.cross(A[:, 2], A[:, 0])
    c2 = np.cross(A[:, 0], A[:, 1])
    det = (A[:, 0] * c0).sum(1)
    g = np.stack([c0, c1, c2], 1) / det[:, None, None]                   # grad lambda_{1..3}
    G = np.concatenate([-g.sum(1, keepdims=True), g], 1)                 # [E, 4, 3]
    vol = np.abs(det)
    Ke = (kappa.astype(L) * vol * w.sum())[:, None, None] * np.einsum("eai,ebi->eab", G, G)
    K = np.zeros((n, n), dtype=L)
    np.add.at(K, (conn[:, :, None], conn[:, None, :]), Ke)
    b = np.zeros(n, dtype=L)
    np.add.at(b, conn, vol[:, None] * (w[:, None] * phi).sum(0)[None, :])
    return K, b


def _fd_loss(mesh, pts, kappa, u_t):
    """Loss of the same discrete model evaluated entirely in extended
    precision (assembly and solve): with eps = 1e-6 the float64 rounding of K
    alone (one ulp of a node's sum over ~24 elements, divided by eps times
    one element's share) would put ~1e-8 of noise into the differences."""
    free = (~mesh.boundary_mask).cpu().numpy()
    K, b = _p1_tet_system_extended(pts.cpu().numpy(), mesh.elements().cpu().numpy(),
                                   kappa.cpu().numpy(), mesh.n_points)
    u = _solve_spd_extended(K[free][:, free], b[free])
    d = u - u_t.cpu().numpy()[free].astype(np.longdouble)
    return (d * d).sum()


def test_adjoint_against_central_differences(cuda):
    """dL/dkappa and dL/dx at 32 seeded elements and 32 seeded node
    coordinates against central differences (eps = 1e-6) of the same
    discrete model, within 1e-8 relative (1e-11 of the largest gradient
    entry for entries near zero)."""
    extended = np.finfo(np.longdouble).eps < 1e-25          # IEEE quad (aarch64)
    tol = 1e-8 if extended else 1e-6
    mesh = tg.gen_unit_cube(5, jitter=0.15, seed=41).to(cuda)
    rng = np.random.default_rng(42)
    kappa0 = torch.from_numpy(rng.lognormal(0.0, 0.5, mesh.n_elements)).to(cuda)
    u_t = torch.from_numpy(rng.uniform(0.0, 0.05, mesh.n_points)).to(cuda)
    asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    src = tg.const_node_assembler(1.0).from_mesh(mesh)
    cond = tg.Condenser(mesh.boundary_mask)
    pts = mesh.points.clone().requires_grad_(True)
    kappa = kappa0.clone().requires_grad_(True)
    u = tg.solve_diffusion(asm, src, cond, pts, kappa, rtol=1e-15)
    loss = ((u - u_t) ** 2)[~mesh.boundary_mask].sum()
    loss.backward()
    eps = 1e-6
    gk = kappa.grad.cpu().numpy()
    gx = pts.grad.cpu().numpy()
    for e in rng.choice(mesh.n_elements, 32, replace=False):
        kp, km = kappa0.clone(), kappa0.clone()
        kp[e] *= 1 + eps
        km[e] *= 1 - eps
        fd = float((_fd_loss(mesh, mesh.points, kp, u_t) - _fd_loss(mesh, mesh.points, km, u_t))
                   / (2 * eps * float(kappa0[e])))
        assert abs(fd - gk[e]) <= tol * abs(fd) + 1e-11 * np.abs(gk).max(), (e, fd, gk[e])
    interior = torch.nonzero(~mesh.boundary_mask).reshape(-1).cpu().numpy()
    for n in rng.choice(interior, 32, replace=False):
        d = int(rng.integers(0, 3))
        pp, pm = mesh.points.clone(), mesh.points.clone()
        pp[n, d] += eps
        pm[n, d] -= eps
        fd = float((_fd_loss(mesh, pp, kappa0, u_t) - _fd_loss(mesh, pm, kappa0, u_t)) / (2 * eps))
        assert abs(fd - gx[n, d]) <= tol * abs(fd) + 1e-11 * np.abs(gx).max(), (n, d, fd, gx[n, d])


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
