"""Meshes with several element types on the GPU: every type assembled by
its kernels, the results summed onto the union pattern (matrices) or the
nodes (load vectors) by one deterministic gather-sum, against the oracle's
per-type assembly summed in type order (1e-12 relative Frobenius)."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import rel_fro
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


def test_mixed_quad_triangle_mesh(cuda):
    m = tg.gen_unit_square_mixed(12, jitter=0.2, seed=41)
    g = m.to(cuda)
    rng = np.random.default_rng(42)
    kappa = {et: torch.from_numpy(rng.lognormal(0.0, 1.0, c.shape[0])) for et, c in m.cells.items()}
    E = {et: torch.from_numpy(rng.uniform(0.5, 2.0, c.shape[0])) for et, c in m.cells.items()}
    f = torch.from_numpy(rng.uniform(-1.0, 1.0, m.n_points))

    asm = tg.LaplaceElementAssembler.from_mesh(g)
    K = asm(g.points, element_data={"kappa": {et: k.to(cuda) for et, k in kappa.items()}})
    edges, Ko = O.assemble_mixed(m.points, m.cells, m.n_points, {
        et: (lambda p, c, et=et: O.element_locals_diffusion(p, c, et, kappa[et], 2)) for et in m.cells})
    assert torch.equal(asm.edges.cpu(), edges)
    assert K.layout_hash == O.layout_hash(edges[0], edges[1])
    assert rel_fro(K.values, Ko) <= 1e-12
    # one tensor over all elements, types concatenated in type order
    flat = torch.cat([kappa[et] for et in m.cells]).to(cuda)
    assert torch.equal(asm(g.points, element_data={"kappa": flat}).values, K.values)

    M = tg.MassElementAssembler.from_assembler(asm)(g.points)
    _, Mo = O.assemble_mixed(m.points, m.cells, m.n_points,
                             {et: (lambda p, c, et=et: O.element_locals_mass(p, c, et, 2)) for et in m.cells})
    assert rel_fro(M.values, Mo) <= 1e-12

    El = tg.LinearElasticityElementAssembler.from_assembler(asm, nu=0.3)(
        g.points, element_data={"E": {et: e.to(cuda) for et, e in E.items()}})
    _, Elo = O.assemble_mixed(m.points, m.cells, m.n_points, {
        et: (lambda p, c, et=et: O.element_locals_elasticity(p, c, et, E[et], 0.3, 2)) for et in m.cells})
    assert rel_fro(El.values, Elo) <= 1e-12

    b = tg.LoadNodeAssembler.from_mesh(g)(g.points, point_data={"f": f.to(cuda)})
    bo = sum(O.assemble_load(m.points, c, et, m.n_points, f_nodes=f) for et, c in m.cells.items())
    assert rel_fro(b, bo) <= 1e-12

    # the assembled system is consistent: a Dirichlet solve of the mixed
    # Poisson problem matches the oracle's
    cond = tg.Condenser(g.boundary_mask)
    Ki, bi = cond(K, b)
    ui, info = tg.pcg_solve(Ki, bi, rtol=1e-13, return_info=True)
    assert info.converged
    uo = O.solve_dirichlet(Ko, edges[0], edges[1], m.n_points, m.boundary_mask, bo)
    assert rel_fro(cond.recover(ui), uo) <= 1e-10


def test_mixed_mesh_gradients(cuda):
    """Gradients on a quad + triangle mesh (each type through its own
    adjoint kernels, summed by the differentiable combine): dL/dpoints and
    dL/dkappa of diffusion (kappa one tensor over all elements), dL/dpoints
    of mass, dL/dE (a per-type dict) and dL/dpoints of elasticity, and
    dL/dpoints, dL/df of the nodal load, against the oracle's per-type
    assembly under autograd."""
    m = tg.gen_unit_square_mixed(6, jitter=0.2, seed=43)
    g = m.to(cuda)
    rng = np.random.default_rng(44)
    types = list(m.cells)
    k0 = torch.from_numpy(rng.lognormal(0.0, 1.0, sum(c.shape[0] for c in m.cells.values())))
    E0 = {et: torch.from_numpy(rng.uniform(0.5, 2.0, c.shape[0])) for et, c in m.cells.items()}
    f0 = torch.from_numpy(rng.uniform(-1.0, 1.0, m.n_points))
    asm = tg.LaplaceElementAssembler.from_mesh(g)
    nnz = asm.edges.shape[1]
    W = torch.from_numpy(rng.uniform(-1.0, 1.0, nnz))
    W3 = torch.from_numpy(rng.uniform(-1.0, 1.0, (nnz, 2, 2)))
    wb = torch.from_numpy(rng.uniform(-1.0, 1.0, m.n_points))

    P = g.points.clone().requires_grad_(True)
    kap = k0.clone().to(cuda).requires_grad_(True)
    Ed = {et: e.clone().to(cuda).requires_grad_(True) for et, e in E0.items()}
    f = f0.clone().to(cuda).requires_grad_(True)
    K = asm(P, element_data={"kappa": kap})
    M = tg.MassElementAssembler.from_assembler(asm)(P)
    El = tg.LinearElasticityElementAssembler.from_assembler(asm, nu=0.3)(P, element_data={"E": Ed})
    b = tg.LoadNodeAssembler.from_mesh(g)(P, point_data={"f": f})
    loss = ((K.values * W.to(cuda)).sum() + (M.values * W.to(cuda)).sum()
            + (El.values.reshape(-1, 2, 2) * W3.to(cuda)).sum() + (b * wb.to(cuda)).sum())
    loss.backward()

    Po = m.points.clone().requires_grad_(True)
    ko = k0.clone().requires_grad_(True)
    Eo = {et: e.clone().requires_grad_(True) for et, e in E0.items()}
    fo = f0.clone().requires_grad_(True)
    kparts, o = {}, 0
    for et in types:
        n = m.cells[et].shape[0]
        kparts[et] = ko[o:o + n]
        o += n
    _, Ko = O.assemble_mixed(Po, m.cells, m.n_points, {
        et: (lambda p, c, et=et: O.element_locals_diffusion(p, c, et, kparts[et], 2)) for et in types})
    _, Mo = O.assemble_mixed(Po, m.cells, m.n_points,
                             {et: (lambda p, c, et=et: O.element_locals_mass(p, c, et, 2)) for et in types})
    _, Elo = O.assemble_mixed(Po, m.cells, m.n_points, {
        et: (lambda p, c, et=et: O.element_locals_elasticity(p, c, et, Eo[et], 0.3, 2)) for et in types})
    bo = sum(O.assemble_load(Po, c, et, m.n_points, f_nodes=fo) for et, c in m.cells.items())
    lo = (Ko * W).sum() + (Mo * W).sum() + (Elo.reshape(-1, 2, 2) * W3).sum() + (bo * wb).sum()
    lo.backward()
    assert abs(float(loss.detach()) - float(lo.detach())) <= 1e-12 * abs(float(lo.detach()))
    assert rel_fro(P.grad.cpu(), Po.grad) <= 1e-10
    assert rel_fro(kap.grad.cpu(), ko.grad) <= 1e-10
    for et in types:
        assert rel_fro(Ed[et].grad.cpu(), Eo[et].grad) <= 1e-10
    assert rel_fro(f.grad.cpu(), fo.grad) <= 1e-10
