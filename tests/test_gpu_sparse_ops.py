"""SparseMatrix arithmetic as the reference's examples use it (time
integrators: ``K = M + dt * D * D * A``, examples/diffusion/heat/heat.py:43;
``SparseMatrix(mat.edata * s, mat.row, mat.col, mat.shape)``,
examples/wave/wave.py:61-63): same-layout sums on the values, different
layouts through the union of the patterns, scalar products and gradients,
against dense arithmetic; then the heat example's implicit Euler steps
against a dense solve."""
import numpy as np
import pytest
import torch

import tensormesh_gb300 as tg
from tensormesh_gb300.sparse import SparseMatrix
from conftest import rel_fro

pytestmark = pytest.mark.gpu


class AAssembler(tg.ElementAssembler):
    def forward(self, gradu, gradv):
        return gradu @ gradv


class MAssembler(tg.ElementAssembler):
    def forward(self, u, v):
        return u * v


def test_same_and_different_layouts(cuda):
    m = tg.gen_unit_square(8, jitter=0.2, seed=81).to(cuda)
    M = MAssembler.from_mesh(m)()
    A = AAssembler.from_mesh(m)()          # its own topology, the same pattern
    dt = 0.01
    K = M + dt * A
    assert torch.equal(K.edges, M.edges)
    assert torch.allclose(K.to_dense(), M.to_dense() + dt * A.to_dense(), rtol=0, atol=1e-15)
    assert torch.allclose((M - A / 2).to_dense(), M.to_dense() - 0.5 * A.to_dense(), rtol=0, atol=1e-15)
    assert torch.allclose((-M).to_dense(), -M.to_dense())
    S = SparseMatrix(M.edata * 3.0, M.row, M.col, M.shape)
    assert torch.allclose(S.to_dense(), 3.0 * M.to_dense())
    # a different pattern: the union
    n = M.shape[0]
    rng = np.random.default_rng(82)
    r = torch.from_numpy(rng.integers(0, n, 40)).to(cuda)
    c = torch.from_numpy(rng.integers(0, n, 40)).to(cuda)
    key = torch.unique(r * n + c)
    P = SparseMatrix(torch.from_numpy(rng.uniform(-1, 1, key.numel())).to(cuda), key // n, key % n, (n, n))
    U = M + P
    assert torch.allclose(U.to_dense(), M.to_dense() + P.to_dense(), rtol=0, atol=1e-15)
    x = torch.from_numpy(rng.uniform(-1, 1, n)).to(cuda)
    assert torch.allclose(U @ x, U.to_dense() @ x, rtol=1e-13, atol=1e-13)
    # gradients flow through the values
    s = torch.tensor(0.3, dtype=torch.float64, device=cuda, requires_grad=True)
    (M + s * A).values.sum().backward()
    assert torch.allclose(s.grad, A.values.sum())


def test_heat_implicit_euler(cuda):
    m = tg.gen_unit_square(12, jitter=0.1, seed=83).to(cuda)
    M = MAssembler.from_mesh(m, quadrature_order=2)()
    A = AAssembler.from_mesh(m, quadrature_order=2)()
    cond = tg.Condenser(m.boundary_mask)
    dt = 5e-3
    K = M + dt * A
    K_ = cond(K)[0]
    x = m.points.double()
    U = torch.sin(np.pi * x[:, 0]) * torch.sin(np.pi * x[:, 1])
    Kd, Md = K.to_dense(), M.to_dense()
    free = ~m.boundary_mask
    Ud = U.clone()
    for _ in range(5):
        U = cond.recover(K_.solve(cond.condense_rhs(M @ U), tol=1e-13))
        F = Md @ Ud
        Ud = torch.zeros_like(Ud)
        Ud[free] = torch.linalg.solve(Kd[free][:, free], F[free])
    assert rel_fro(U, Ud) <= 1e-10
