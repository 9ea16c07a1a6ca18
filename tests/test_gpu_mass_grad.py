"""Gradients of a P1 mass matrix with respect to the node coordinates and
its scalar density (``MassAssembly``: the ``tm_adjoint_p1`` kernel in its
mass mode) against the oracle's autograd through the reference's op
sequence (gather, Jacobian, det, quadrature einsum, index_add_), on
triangles and tetrahedra, within 1e-10 relative."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import rel_fro
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("etype", ["triangle", "tetra"])
def test_mass_gradients_match_oracle_autograd(etype, cuda):
    mesh = (tg.gen_unit_square(9, jitter=0.2, seed=91) if etype == "triangle"
            else tg.gen_unit_cube(4, jitter=0.2, seed=92))
    rng = np.random.default_rng(93)
    gm = mesh.to(cuda)
    asm = tg.MassElementAssembler.from_mesh(gm)
    nnz = asm.edges.shape[1]
    w = torch.from_numpy(rng.uniform(-1.0, 1.0, nnz))
    rho0 = 1.7
    pts = gm.points.clone().requires_grad_(True)
    rho = torch.tensor(rho0, dtype=torch.float64, device=cuda, requires_grad=True)
    M = asm(pts, scalar_data={"rho": rho})
    (M.values * w.to(cuda)).sum().backward()

    P = mesh.points.clone().requires_grad_(True)
    conn = mesh.elements().long()
    edges, _, Mo = O.assemble_matrix(P, conn, mesh.n_points, lambda p, c: O.element_locals_mass(p, c, etype, 2))
    assert torch.equal(asm.edges.cpu(), edges)
    ro = torch.tensor(rho0, dtype=torch.float64, requires_grad=True)
    ((ro * Mo) * w).sum().backward()
    assert rel_fro(M.values.detach().cpu(), rho0 * Mo.detach()) <= 1e-12
    assert rel_fro(pts.grad.cpu(), P.grad) <= 1e-10
    assert abs(float(rho.grad) - float(ro.grad)) <= 1e-12 * abs(float(ro.grad))


def test_mass_gradient_without_density(cuda):
    mesh = tg.gen_unit_cube(3, jitter=0.2, seed=94)
    gm = mesh.to(cuda)
    asm = tg.MassElementAssembler.from_mesh(gm)
    w = torch.from_numpy(np.random.default_rng(95).uniform(-1.0, 1.0, asm.edges.shape[1]))
    pts = gm.points.clone().requires_grad_(True)
    (asm(pts).values * w.to(cuda)).sum().backward()
    P = mesh.points.clone().requires_grad_(True)
    _, _, Mo = O.assemble_matrix(P, mesh.elements().long(), mesh.n_points,
                                 lambda p, c: O.element_locals_mass(p, c, "tetra", 2))
    (Mo * w).sum().backward()
    assert rel_fro(pts.grad.cpu(), P.grad) <= 1e-10
