"""P2 tetrahedral linear elasticity with the bottom face clamped and a body
force (0, 0, -1): block-aware condensation and block-CSR Jacobi-PCG.
Small case against a SciPy direct solve of the oracle's system (1e-9
relative); full size (32^3 x 6 P2 tets) to 1e-10 relative residual, with the
true residual recomputed by an independent SpMV."""
import numpy as np
import pytest
import scipy.sparse
import scipy.sparse.linalg
import torch

import tensormesh_gb300 as tg
from conftest import rel_fro
from oracle import fem_oracle as O
from tensormesh_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _problem(mesh, E, dev):
    m = mesh.to(dev)
    asm = tg.LinearElasticityElementAssembler.from_mesh(m, nu=0.3)
    K = asm(m.points, element_data={"E": E.to(dev)})
    load = tg.const_node_assembler(torch.tensor([0.0, 0.0, -1.0])).from_mesh(m)
    b = load(m.points)
    clamp = (m.points[:, 2] == 0.0).repeat_interleave(3)
    return m, K, b, clamp


def test_small_elasticity_solve_matches_direct(cuda):
    mesh = tg.gen_unit_cube(3, order=2)
    E = torch.from_numpy(np.random.default_rng(61).uniform(0.5, 2.0, mesh.n_elements))
    m, K, b, clamp = _problem(mesh, E, cuda)
    cond = tg.Condenser(clamp)
    Kc, bc = cond(K, b)
    assert Kc._block == 3                        # condensed as 3x3 blocks
    uc, info = tg.pcg_solve(Kc, bc, rtol=1e-13, return_info=True)
    assert info.converged
    u = cond.recover(uc).cpu()
    # oracle: assembly, then SciPy direct solve of the condensed system
    _, _, Ko = O.assemble_matrix(mesh.points, mesh.elements(), mesh.n_points,
                                 lambda p, c, E: O.element_locals_elasticity(p, c, "tetra10", E, 0.3, 2), E=E)
    edges, _ = O.element_pattern(mesh.elements(), mesh.n_points)
    r, c = O.block_coo_indices(edges[0], edges[1], 3)
    A = scipy.sparse.coo_matrix((Ko.reshape(-1).numpy(), (r.numpy(), c.numpy())),
                                shape=(3 * mesh.n_points,) * 2).tocsr()
    bo = O.assemble_load(mesh.points, mesh.elements(), "tetra10", mesh.n_points, const=1.0)
    rhs = torch.zeros(mesh.n_points, 3, dtype=torch.float64)
    rhs[:, 2] = -bo
    free = ~clamp.cpu().numpy()
    uo = np.zeros(3 * mesh.n_points)
    uo[free] = scipy.sparse.linalg.spsolve(A[free][:, free].tocsc(), rhs.reshape(-1).numpy()[free])
    assert rel_fro(b.cpu(), rhs.reshape(-1)) <= 1e-12
    assert rel_fro(u, torch.from_numpy(uo)) <= 1e-9


def test_full_size_elasticity_pcg(cuda):
    wl = W.elasticity_p2tet(32)
    m, K, b, clamp = _problem(wl.mesh, wl.data["E"], cuda)
    assert K.nnz == 69108489
    cond = tg.Condenser(clamp)
    Kc, bc = cond(K, b)
    uc, info = tg.pcg_solve(Kc, bc, rtol=1e-10, max_iter=50000, check_every=100, return_info=True)
    assert info.converged, info
    res = float((bc - Kc @ uc).norm() / bc.norm())
    assert res <= 2e-10, res
    u = cond.recover(uc)
    assert float(u[2::3].min()) < 0.0               # the body sags under (0, 0, -1)
