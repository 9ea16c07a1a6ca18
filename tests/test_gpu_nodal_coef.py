"""A per-node coefficient given as point_data to a recognised form, as the
reference's coefficient-identification example passes it
(examples/inverse_design/coefficient_identification.py:49-79: a
``WeightedLaplace`` form ``kappa * (gradu @ gradv)`` with ``point_data=
{"kappa": kappa}``, condensation, ``.solve``, ``recover``, a least-squares
loss and ``backward``): values and the gradient with respect to the
unconstrained parameter against the same chain through the oracle's op
sequence (nodal kappa interpolated at the quadrature points) and a dense
solve."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from conftest import rel_fro
from oracle import fem_oracle as O

pytestmark = pytest.mark.gpu


class WeightedLaplace(tg.ElementAssembler):
    def forward(self, gradu, gradv, kappa):
        return kappa * (gradu @ gradv)


class Source(tg.NodeAssembler):
    def forward(self, v, f):
        return v * f


def _oracle_K(points, conn, n, kappa_nodes, etype):
    grad, jxw = O.shape_grad_jxw(points, conn, etype, 2)
    _, phi, _ = O.shape_tables(etype, 2)
    kq = kappa_nodes[conn] @ phi.T                                   # nodal data at the points
    Ke = torch.einsum("eq,eqid,eqjd,eq->eij", kq, grad, grad, jxw)
    edges, slot = O.element_pattern(conn, n)
    return edges, O.reduce_project(slot, Ke.reshape(-1), edges.shape[1])


@pytest.mark.parametrize("etype", ["triangle", "tetra"])
def test_nodal_coefficient_chain(etype, cuda):
    mesh = tg.gen_unit_square(10, jitter=0.2, seed=71) if etype == "triangle" else tg.gen_unit_cube(4, jitter=0.2, seed=72)
    n = mesh.n_points
    rng = np.random.default_rng(73)
    theta0 = torch.from_numpy(rng.uniform(-0.5, 0.5, n))
    u_obs = torch.from_numpy(rng.uniform(0.0, 0.05, n))
    f = torch.ones(n, dtype=torch.float64)

    gm = mesh.to(cuda)
    cond = tg.Condenser(gm.boundary_mask)
    theta = theta0.clone().to(cuda).requires_grad_(True)
    kappa = 1.0 + torch.tanh(theta)
    K = WeightedLaplace.from_mesh(gm)(point_data={"kappa": kappa}).double()
    b = Source.from_mesh(gm)(point_data={"f": f.to(cuda)}).double()
    K_, b_ = cond(K, b)
    u = cond.recover(K_.solve(b_, tol=1e-13))
    loss = ((u - u_obs.to(cuda)) ** 2).sum()
    loss.backward()

    to = theta0.clone().requires_grad_(True)
    ko = 1.0 + torch.tanh(to)
    conn = mesh.elements().long()
    edges, Ko = _oracle_K(mesh.points, conn, n, ko, etype)
    assert torch.equal(K.edges.cpu(), edges)
    assert rel_fro(K.values.detach().cpu(), Ko.detach()) <= 1e-12
    bo = O.assemble_load(mesh.points, conn, etype, n, f_nodes=f)
    Kd = torch.zeros(n, n, dtype=torch.float64).index_put((edges[0].long(), edges[1].long()), Ko, accumulate=True)
    free = torch.nonzero(~mesh.boundary_mask).reshape(-1)
    uo = torch.zeros(n, dtype=torch.float64)
    uo = uo.index_put((free,), torch.linalg.solve(Kd[free][:, free], bo[free]))
    ((uo - u_obs) ** 2).sum().backward()
    assert rel_fro(u.detach().cpu(), uo.detach()) <= 1e-10
    assert rel_fro(theta.grad.cpu(), to.grad) <= 1e-8


def test_nodal_coefficient_unsupported_cases(cuda):
    m = tg.gen_unit_square(3, order=2, jitter=0.1, seed=74).to(cuda)
    with pytest.raises(NotImplementedError):
        WeightedLaplace.from_mesh(m)(point_data={"kappa": torch.ones(m.n_points, dtype=torch.float64, device=cuda)})
