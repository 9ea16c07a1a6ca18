"""Differentiable sparse products: y = A @ x with x and A's values requiring
grad (the reference's SparseMatrix product is a torch sparse product, and
its physics-informed example trains a network through ``K_ @ U``),
against dense torch autograd of the same matrices, scalar and 3x3-block;
and a residual loss through assembly, condensation and the product back to
kappa, against the oracle's assembly under autograd."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import rel_fro
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


def _dense(A):
    return A.to_dense().detach().cpu()


def test_matvec_gradients_scalar_and_block(cuda):
    mesh = tg.gen_unit_square(12, jitter=0.2, seed=81).to(cuda)
    rng = np.random.default_rng(82)
    kap = torch.from_numpy(rng.lognormal(0.0, 1.0, mesh.n_elements)).to(cuda)
    K = tg.LaplaceElementAssembler.from_mesh(mesh)(mesh.points, element_data={"kappa": kap})
    E = tg.LinearElasticityElementAssembler.from_mesh(mesh)(mesh.points)
    for A in (K, E):
        n = A.shape[0]
        x0 = torch.from_numpy(rng.uniform(-1.0, 1.0, n))
        w = torch.from_numpy(rng.uniform(-1.0, 1.0, n))
        vals = A.values.detach().clone().requires_grad_(True)
        Av = A.with_values(vals)
        x = x0.clone().to(cuda).requires_grad_(True)
        y = Av @ x
        (y * w.to(cuda)).sum().backward()
        Ad = _dense(A)
        assert rel_fro(y.detach().cpu(), Ad @ x0) <= 1e-14
        assert rel_fro(x.grad.cpu(), Ad.T @ w) <= 1e-14
        # dL/dA_ij = w_i x_j at the stored entries
        gv = vals.grad.detach().cpu().reshape(-1)
        want = w[A.row_indices.cpu()] * x0[A.col_indices.cpu()]
        assert rel_fro(gv, want) <= 1e-14
        # a second backward reuses the transpose's cached CSR view
        x2 = x0.clone().to(cuda).requires_grad_(True)
        w2 = torch.from_numpy(rng.uniform(-1.0, 1.0, n))
        ((Av @ x2) * w2.to(cuda)).sum().backward()
        assert rel_fro(x2.grad.cpu(), Ad.T @ w2) <= 1e-14
    # a non-symmetric matrix: the transpose matters
    S = K + K.with_values(torch.from_numpy(rng.uniform(0.0, 1.0, K.nnz)).to(cuda))
    x = torch.from_numpy(rng.uniform(-1.0, 1.0, S.shape[0])).to(cuda).requires_grad_(True)
    w = torch.from_numpy(rng.uniform(-1.0, 1.0, S.shape[0]))
    ((S @ x).cpu() * w).sum().backward()
    assert rel_fro(x.grad.cpu(), _dense(S).T @ w) <= 1e-14


def test_matmul_of_network_output(cuda):
    """The physics-informed pattern: loss = ||K_ U - F_||^2 with U the output
    of a small network, [n, 1]; the parameters' gradients equal those of the
    dense product."""
    mesh = tg.gen_unit_square(10, jitter=0.1, seed=83).to(cuda)
    K = tg.LaplaceElementAssembler.from_mesh(mesh)(mesh.points)
    M = tg.MassElementAssembler.from_mesh(mesh)(mesh.points)
    f = torch.ones(mesh.n_points, dtype=torch.float64, device=cuda)
    F = M @ f
    Kc, Fc = tg.Condenser(mesh.boundary_mask)(K, F)
    coords = mesh.points[~mesh.boundary_mask]
    torch.manual_seed(0)
    net = torch.nn.Sequential(torch.nn.Linear(2, 16), torch.nn.Tanh(), torch.nn.Linear(16, 1)).double().to(cuda)
    loss = ((Kc @ net(coords) - Fc[:, None]) ** 2).sum()
    loss.backward()
    g = [p.grad.detach().clone() for p in net.parameters()]
    net.zero_grad()
    Kd = Kc.to_dense().to(cuda)
    loss_d = ((Kd @ net(coords) - Fc[:, None]) ** 2).sum()
    loss_d.backward()
    assert abs(float(loss.detach()) - float(loss_d.detach())) <= 1e-12 * float(loss_d.detach())
    for a, p in zip(g, net.parameters()):
        assert rel_fro(a, p.grad) <= 1e-12


def test_residual_loss_back_to_kappa(cuda):
    """L = ||K(kappa)_ii u - b_i||^2 for a fixed u: dL/dkappa through the
    product's values gradient, the condensation and the assembly adjoint,
    against the oracle's assembly under autograd with a dense product."""
    mesh = tg.gen_unit_square(8, jitter=0.2, seed=84)
    rng = np.random.default_rng(85)
    k0 = torch.from_numpy(rng.lognormal(0.0, 0.5, mesh.n_elements))
    u0 = torch.from_numpy(rng.uniform(-1.0, 1.0, mesh.n_points))
    gm = mesh.to(cuda)
    kap = k0.clone().to(cuda).requires_grad_(True)
    K = tg.LaplaceElementAssembler.from_mesh(gm)(gm.points, element_data={"kappa": kap})
    r = K @ u0.to(cuda)
    loss = (r ** 2).sum()
    loss.backward()
    ko = k0.clone().requires_grad_(True)
    edges, _, Ko = O.assemble_matrix(mesh.points, mesh.elements(), mesh.n_points,
                                     lambda p, c, kappa: O.element_locals_diffusion(p, c, "triangle", kappa, 2),
                                     kappa=ko)
    Kd = torch.zeros(mesh.n_points, mesh.n_points, dtype=torch.float64).index_put(
        (edges[0].long(), edges[1].long()), Ko, accumulate=True)
    lo = ((Kd @ u0) ** 2).sum()
    lo.backward()
    assert abs(float(loss.detach()) - float(lo.detach())) <= 1e-12 * float(lo.detach())
    assert rel_fro(kap.grad.cpu(), ko.grad) <= 1e-10


def test_fused_assembly_with_gradients(cuda):
    """assemble_forms with a coefficient requiring grad runs each form's
    differentiable call: the same values, gradients equal to the
    assemblers' own."""
    mesh = tg.gen_unit_cube(3, jitter=0.2, seed=87).to(cuda)
    rng = np.random.default_rng(88)
    k0 = torch.from_numpy(rng.lognormal(0.0, 1.0, mesh.n_elements)).to(cuda)
    K_asm = tg.LaplaceElementAssembler.from_mesh(mesh)
    M_asm = tg.MassElementAssembler.from_assembler(K_asm)
    W = torch.from_numpy(rng.uniform(-1.0, 1.0, K_asm.edges.shape[1])).to(cuda)
    with torch.no_grad():
        K0, M0 = tg.assemble_forms([K_asm, M_asm], mesh.points, {"kappa": k0})
    k1 = k0.clone().requires_grad_(True)
    K1, M1 = tg.assemble_forms([K_asm, M_asm], mesh.points, {"kappa": k1})
    assert rel_fro(K1.detach(), K0) <= 1e-13 and rel_fro(M1.detach(), M0) <= 1e-13
    ((K1 + M1) * W).sum().backward()
    k2 = k0.clone().requires_grad_(True)
    (K_asm(mesh.points, element_data={"kappa": k2}).values * W).sum().backward()
    assert rel_fro(k1.grad, k2.grad) <= 1e-14
