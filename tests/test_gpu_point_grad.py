"""Gradients of diffusion and mass matrices with respect to the node
coordinates (and kappa) on elements whose Jacobian varies -- P2 triangles
and tetrahedra, Q1 and Q2 quadrilaterals -- through ``tm_adjoint_general``
(per quadrature point: dL/dJ_q from dL/dvalues, spread to the nodes with
the reference gradients), against the oracle's autograd through the
reference's op sequence, within 1e-10 relative."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import rel_fro
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu

MESHES = {
    "triangle6": lambda: tg.gen_unit_square(3, order=2, jitter=0.1, seed=91),
    "tetra10": lambda: tg.gen_unit_cube(2, order=2, jitter=0.1, seed=92),
    "quad": lambda: tg.gen_unit_square(4, jitter=0.2, seed=93, cell="quad"),
    "quad9": lambda: tg.gen_unit_square(3, order=2, jitter=0.1, seed=94, cell="quad"),
}


@pytest.mark.parametrize("etype", list(MESHES))
def test_point_and_kappa_gradients(etype, cuda):
    mesh = MESHES[etype]()
    rng = np.random.default_rng(95)
    k0 = torch.from_numpy(rng.lognormal(0.0, 0.5, mesh.n_elements))
    gm = mesh.to(cuda)
    K_asm = tg.DiffusionElementAssembler.from_mesh(gm)
    M_asm = tg.MassElementAssembler.from_assembler(K_asm)
    nnz = K_asm.edges.shape[1]
    wk = torch.from_numpy(rng.uniform(-1.0, 1.0, nnz))
    wm = torch.from_numpy(rng.uniform(-1.0, 1.0, nnz))
    pts = gm.points.clone().requires_grad_(True)
    kap = k0.clone().to(cuda).requires_grad_(True)
    K = K_asm(pts, element_data={"kappa": kap})
    M = M_asm(pts, scalar_data={"rho": 1.3})
    ((K.values * wk.to(cuda)).sum() + (M.values * wm.to(cuda)).sum()).backward()

    P = mesh.points.clone().requires_grad_(True)
    ko = k0.clone().requires_grad_(True)
    conn = mesh.elements().long()
    _, _, Ko = O.assemble_matrix(P, conn, mesh.n_points,
                                 lambda p, c, kappa: O.element_locals_diffusion(p, c, etype, kappa, 2), kappa=ko)
    _, _, Mo = O.assemble_matrix(P, conn, mesh.n_points, lambda p, c: O.element_locals_mass(p, c, etype, 2))
    assert rel_fro(K.values.detach().cpu(), Ko.detach()) <= 1e-12
    ((Ko * wk).sum() + (1.3 * Mo * wm).sum()).backward()
    assert rel_fro(pts.grad.cpu(), P.grad) <= 1e-10
    assert rel_fro(kap.grad.cpu(), ko.grad) <= 1e-10
