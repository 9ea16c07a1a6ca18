"""Gradients of isotropic elasticity matrices with respect to the modulus
(``ElasticityAssembly``: the ``tm_coef_grad`` kernel), and of diffusion
matrices with respect to their coefficient on every element type, against the
oracle's autograd through the reference's op sequence (Voigt B^T C B,
quadrature einsum, index_add_), for every element type, within 1e-10
relative; and the reference's compliance-minimisation workflow (a SIMP
plane-stress form, Dirichlet condensation, solve, compliance, backward)
against the same chain through the oracle and a dense solve."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import rel_fro
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu

MESHES = {
    "triangle": lambda: tg.gen_unit_square(6, jitter=0.2, seed=61),
    "tetra": lambda: tg.gen_unit_cube(3, jitter=0.2, seed=62),
    "triangle6": lambda: tg.gen_unit_square(3, order=2, jitter=0.1, seed=63),
    "tetra10": lambda: tg.gen_unit_cube(2, order=2, jitter=0.1, seed=64),
    "quad": lambda: tg.gen_unit_square(4, jitter=0.2, seed=65, cell="quad"),
    "quad9": lambda: tg.gen_unit_square(3, order=2, jitter=0.1, seed=66, cell="quad"),
}


@pytest.mark.parametrize("etype", list(MESHES))
def test_young_gradient_matches_oracle_autograd(etype, cuda):
    mesh = MESHES[etype]()
    rng = np.random.default_rng(67)
    E0 = torch.from_numpy(rng.uniform(0.5, 2.0, mesh.n_elements))
    gm = mesh.to(cuda)
    asm = tg.LinearElasticityElementAssembler.from_mesh(gm, nu=0.3)
    D = mesh.points.shape[1]
    W = torch.from_numpy(rng.uniform(-1.0, 1.0, (asm.edges.shape[1], D, D)))
    E = E0.clone().to(cuda).requires_grad_(True)
    K = asm(gm.points, element_data={"E": E})
    vals = K.values.reshape(-1, D, D)
    (vals * W.to(cuda)).sum().backward()
    Eo = E0.clone().requires_grad_(True)
    conn = mesh.elements().long()
    _, _, Ko = O.assemble_matrix(mesh.points, conn, mesh.n_points,
                                 lambda p, c, E: O.element_locals_elasticity(p, c, etype, E, 0.3, 2), E=Eo)
    assert rel_fro(vals.detach().cpu(), Ko.detach()) <= 1e-12
    (Ko * W).sum().backward()
    assert rel_fro(E.grad.cpu(), Eo.grad) <= 1e-10


@pytest.mark.parametrize("etype", list(MESHES))
@pytest.mark.parametrize("per_element", [True, False])
def test_point_gradient_matches_oracle_autograd(etype, per_element, cuda):
    """dL/dpoints of L = sum W : K(points, E) (the elasticity mode of
    ``tm_adjoint_general``) together with dL/dE, against the oracle's
    autograd, per-element and scalar modulus."""
    mesh = MESHES[etype]()
    rng = np.random.default_rng(69)
    E0 = torch.from_numpy(rng.uniform(0.5, 2.0, mesh.n_elements)) if per_element else torch.tensor(1.7,
                                                                                                  dtype=torch.float64)
    gm = mesh.to(cuda)
    asm = tg.LinearElasticityElementAssembler.from_mesh(gm, nu=0.27)
    D = mesh.points.shape[1]
    W = torch.from_numpy(rng.uniform(-1.0, 1.0, (asm.edges.shape[1], D, D)))
    P = gm.points.clone().requires_grad_(True)
    E = E0.clone().to(cuda).requires_grad_(True)
    K = asm(P, element_data={"E": E}) if per_element else asm(P, scalar_data={"E": E})
    vals = K.values.reshape(-1, D, D)
    (vals * W.to(cuda)).sum().backward()
    Po = mesh.points.clone().requires_grad_(True)
    Eo = E0.clone().requires_grad_(True)
    Ef = Eo if per_element else Eo.expand(mesh.n_elements)
    conn = mesh.elements().long()
    _, _, Ko = O.assemble_matrix(Po, conn, mesh.n_points,
                                 lambda p, c, E: O.element_locals_elasticity(p, c, etype, E, 0.27, 2), E=Ef)
    assert rel_fro(vals.detach().cpu(), Ko.detach()) <= 1e-12
    (Ko * W).sum().backward()
    assert rel_fro(P.grad.cpu(), Po.grad) <= 1e-10
    assert rel_fro(E.grad.cpu(), Eo.grad) <= 1e-10


@pytest.mark.parametrize("etype", ["triangle", "tetra10", "quad9"])
def test_poisson_ratio_gradient_matches_oracle_autograd(etype, cuda):
    """dL/dnu (and dL/dE, dL/dpoints in the same backward) of L = sum W :
    K(points, E, nu) with nu = 0.27 passed as a tensor in scalar_data,
    against the oracle's autograd through its Voigt C(E, nu)."""
    mesh = MESHES[etype]()
    rng = np.random.default_rng(71)
    E0 = torch.from_numpy(rng.uniform(0.5, 2.0, mesh.n_elements))
    gm = mesh.to(cuda)
    asm = tg.LinearElasticityElementAssembler.from_mesh(gm)
    D = mesh.points.shape[1]
    W = torch.from_numpy(rng.uniform(-1.0, 1.0, (asm.edges.shape[1], D, D)))
    P = gm.points.clone().requires_grad_(True)
    E = E0.clone().to(cuda).requires_grad_(True)
    nu = torch.tensor(0.27, dtype=torch.float64, requires_grad=True)
    K = asm(P, element_data={"E": E}, scalar_data={"nu": nu})
    vals = K.values.reshape(-1, D, D)
    (vals * W.to(cuda)).sum().backward()
    Po = mesh.points.clone().requires_grad_(True)
    Eo = E0.clone().requires_grad_(True)
    nuo = torch.tensor(0.27, dtype=torch.float64, requires_grad=True)
    _, _, Ko = O.assemble_matrix(Po, mesh.elements().long(), mesh.n_points,
                                 lambda p, c, E: O.element_locals_elasticity(p, c, etype, E, nuo, 2), E=Eo)
    assert rel_fro(vals.detach().cpu(), Ko.detach()) <= 1e-12
    (Ko * W).sum().backward()
    assert abs(float(nu.grad) - float(nuo.grad)) <= 1e-10 * abs(float(nuo.grad))
    assert rel_fro(E.grad.cpu(), Eo.grad) <= 1e-10
    assert rel_fro(P.grad.cpu(), Po.grad) <= 1e-10


def test_point_gradient_constant_modulus(cuda):
    """Points alone requiring grad, the modulus a plain number of the
    assembler (E = 3, nu = 0.2)."""
    mesh = MESHES["tetra"]()
    gm = mesh.to(cuda)
    asm = tg.LinearElasticityElementAssembler.from_mesh(gm, E=3.0, nu=0.2)
    rng = np.random.default_rng(70)
    W = torch.from_numpy(rng.uniform(-1.0, 1.0, (asm.edges.shape[1], 3, 3)))
    P = gm.points.clone().requires_grad_(True)
    vals = asm(P).values.reshape(-1, 3, 3)
    (vals * W.to(cuda)).sum().backward()
    Po = mesh.points.clone().requires_grad_(True)
    conn = mesh.elements().long()
    Ef = torch.full((mesh.n_elements,), 3.0, dtype=torch.float64)
    _, _, Ko = O.assemble_matrix(Po, conn, mesh.n_points,
                                 lambda p, c, E: O.element_locals_elasticity(p, c, "tetra", E, 0.2, 2), E=Ef)
    (Ko * W).sum().backward()
    assert rel_fro(P.grad.cpu(), Po.grad) <= 1e-10


class SIMPElastic(tg.ElementAssembler):
    """The plane-stress SIMP form of the reference's compliance example
    (examples/inverse_design/compliance_topology.py:31-110), restated."""

    def __post_init__(self, E_max=70e3, E_min=70.0, nu=0.3, penal=3.0):
        self.E_max, self.E_min, self.nu, self.penal = E_max, E_min, nu, penal

    def forward(self, gradu, gradv, rho):
        E = self.E_min + (rho ** self.penal) * (self.E_max - self.E_min)
        d11, d12, d33 = E / (1 - self.nu ** 2), self.nu * E / (1 - self.nu ** 2), E / (2 * (1 + self.nu))
        ux, uy, vx, vy = gradu[0], gradu[1], gradv[0], gradv[1]
        return torch.stack([torch.stack([d11 * ux * vx + d33 * uy * vy, d12 * ux * vy + d33 * uy * vx]),
                            torch.stack([d12 * uy * vx + d33 * ux * vy, d11 * uy * vy + d33 * ux * vx])])


def test_simp_compliance_gradient(cuda):
    """K(rho) of the SIMP form, the left edge clamped, a load on the right
    edge, u = K_ii^-1 F_i, compliance F . u; dC/drho through the library
    (coefficient map, elasticity gradient kernel, differentiable condensation
    and solve) against autograd through the oracle's assembly and a dense
    solve."""
    mesh = tg.gen_unit_square(6, jitter=0.0, seed=0, cell="quad")
    rng = np.random.default_rng(68)
    rho0 = torch.from_numpy(rng.uniform(0.3, 1.0, mesh.n_elements))
    pts = mesh.points
    clamp = (pts[:, 0] == 0.0).repeat_interleave(2)
    F = torch.zeros(2 * mesh.n_points, dtype=torch.float64)
    right = torch.nonzero(pts[:, 0] == 1.0).reshape(-1)
    F[2 * right + 1] = -1.0
    gm = mesh.to(cuda)
    asm = SIMPElastic.from_mesh(gm)
    rho = rho0.clone().to(cuda).requires_grad_(True)
    K = asm(gm.points, element_data={"rho": rho})
    cond = tg.Condenser(clamp.to(cuda))
    Kc, Fc = cond(K, F.to(cuda))
    u = Kc.solve(Fc, backend="scipy")
    (Fc * u).sum().backward()

    ro = rho0.clone().requires_grad_(True)
    E = 70.0 + ro ** 3 * (70e3 - 70.0)
    nu = 0.3 / 1.3
    conn = mesh.elements().long()
    edges, _, Ko = O.assemble_matrix(pts, conn, mesh.n_points,
                                     lambda p, c, E: O.element_locals_elasticity(p, c, "quad", E * 1.6 / 1.69, nu, 2),
                                     E=E)
    n = 2 * mesh.n_points
    r = (2 * edges[0].long()[:, None, None] + torch.arange(2)[None, :, None]).expand(-1, 2, 2).reshape(-1)
    c = (2 * edges[1].long()[:, None, None] + torch.arange(2)[None, None, :]).expand(-1, 2, 2).reshape(-1)
    Kd = torch.zeros(n, n, dtype=torch.float64).index_put((r, c), Ko.reshape(-1), accumulate=True)
    free = torch.nonzero(~clamp).reshape(-1)
    uo = torch.linalg.solve(Kd[free][:, free], F[free])
    (F[free] * uo).sum().backward()
    assert rel_fro(u.detach().cpu(), uo.detach()) <= 1e-8
    assert rel_fro(rho.grad.cpu(), ro.grad) <= 1e-7


class ExpDiffusion(tg.ElementAssembler):
    def forward(self, gradu, gradv, s):
        return torch.exp(s) * (gradu @ gradv)


@pytest.mark.parametrize("etype", list(MESHES))
def test_diffusion_coefficient_gradient_every_element(etype, cuda):
    """dL/dkappa per element on every element type (tm_coef_grad for P2 and
    quadrilaterals, the P1 adjoint kernel for P1), and through a nonlinear
    coefficient map (kappa = exp(s)), against the oracle's autograd."""
    mesh = MESHES[etype]()
    rng = np.random.default_rng(69)
    s0 = torch.from_numpy(rng.uniform(-0.5, 0.5, mesh.n_elements))
    gm = mesh.to(cuda)
    asm = ExpDiffusion.from_mesh(gm)
    W = torch.from_numpy(rng.uniform(-1.0, 1.0, asm.edges.shape[1]))
    s = s0.clone().to(cuda).requires_grad_(True)
    K = asm(gm.points, element_data={"s": s})
    (K.values * W.to(cuda)).sum().backward()
    so = s0.clone().requires_grad_(True)
    _, _, Ko = O.assemble_matrix(mesh.points, mesh.elements().long(), mesh.n_points,
                                 lambda p, c, kappa: O.element_locals_diffusion(p, c, etype, kappa, 2),
                                 kappa=torch.exp(so))
    assert rel_fro(K.values.detach().cpu(), Ko.detach()) <= 1e-12
    (Ko * W).sum().backward()
    assert rel_fro(s.grad.cpu(), so.grad) <= 1e-10
    # a scalar coefficient tensor
    k = torch.tensor(1.3, dtype=torch.float64, device=cuda, requires_grad=True)
    K2 = tg.LaplaceElementAssembler.from_assembler(asm)(gm.points, scalar_data={"kappa": k})
    (K2.values * W.to(cuda)).sum().backward()
    _, _, K1 = O.assemble_matrix(mesh.points, mesh.elements().long(), mesh.n_points,
                                 lambda p, c: O.element_locals_diffusion(p, c, etype, None, 2))
    assert abs(float(k.grad) - float((K1 * W).sum())) <= 1e-10 * abs(float((K1 * W).sum()))
